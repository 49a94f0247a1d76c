// Force walks fused with the integration step (sm_103a, FP32 FMA + MUFU rsqrt;
// no tensor cores: the walk is not a dense contraction).
//
// Both walks give one warp a group of up to 32 consecutive bodies in key order
// (the reference's warp, kernels.cu:342-362) and keep the warp's traversal
// state in shared memory.
//
// k_walk_vote  REFERENCE mode.  A cell is approximated iff all lanes vote
//              dp <= r (kernels.cu:395-406), i.e. iff dp <= min_b r_b over the
//              group; bodies always interact.  Lanes decide up to 32 stack
//              nodes at once and stage the interactions, 32 at a time.  The
//              interaction set is the reference's; only the summation order
//              differs.  Without output positions (out.x null) it writes only
//              the accelerations, in the caller's order (the drop-in's
//              CalculateForces).
// k_walk_acc   PLAIN / MIXED modes.  Lanes test up to 32 stack nodes at once
//              against the group (geometric rule on the group's nearest body,
//              relative rule on its |a_old|); accepted cells and the bodies of
//              opened leaves go to shared-memory lists which are flushed 32
//              entries at a time as dense quadrupole / body-body interactions
//              (every lane computes its body against every entry).  The main
//              pass starts each group from its super-group's shared frontier
//              (k_frontier) and hands out the heaviest groups first.
#pragma once

#include "bh_device.cuh"

namespace ssg {

struct WalkIn {
    const float *x, *y, *vx, *vy, *m, *xlo, *ylo;
    const int* id;
    float* amag;       // |a| of the previous step; written by the bootstrap pass
    const int* gcost;  // the previous step's walk-group cost of each body (accuracy modes)
};
struct WalkOut {
    float *x, *y, *vx, *vy, *m, *xlo, *ylo;
    int* id;
    float *ax, *ay;
    float* amag;  // |a| of this step, for the next step's relative rule
    int* gcost;   // this step's walk-group cost (interaction entries) of each body
    int* box_next;  // [4 nseg] the next step's box (order-preserving ints), folded by the
                    // integrating passes; null: not folded
};

// The next step's bounding box, folded into the integration (the positions a
// walk writes are the next step's).  After each group a warp reduces its new
// positions' box (from the origin, as the box kernel starts: kernels.cu:54-57)
// with shuffles into a per-warp box in shared memory (a float4 and the
// system it belongs to, no registers held across the walk); when the system
// changes and at the warp's end, the box goes to box_next[4 seg] with one
// atomicMin / atomicMax per value that would move it.  Min and max are exact,
// so the box is the box kernel's over the same positions.  A non-finite
// position raises ST_NONFINITE, as the box kernel would in the next step.
struct BoxFold {
    float4* box;  // shared: this warp's box (l, r, b, t)
    int* seg;     // shared: its system, -1: none
    int* box_next;
    int* status;

    __device__ __forceinline__ void init() const {
        if ((threadIdx.x & 31) == 0) {
            *box = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            *seg = -1;
        }
        __syncwarp();
    }
    // lane 0
    __device__ __forceinline__ void publish(int sg, float4 v) const {
        int* bo = box_next + 4 * sg;
        const int4 cur = __ldcg(reinterpret_cast<const int4*>(bo));  // may be stale: only skips
        if (f2ord(v.x) < cur.x) atomicMin(bo + 0, f2ord(v.x));
        if (f2ord(v.y) > cur.y) atomicMax(bo + 1, f2ord(v.y));
        if (f2ord(v.z) < cur.z) atomicMin(bo + 2, f2ord(v.z));
        if (f2ord(v.w) > cur.w) atomicMax(bo + 3, f2ord(v.w));
    }
    // whole warp, after a group of system sg: (l, r, b, t) is this lane's new
    // positions' box from the origin
    __device__ __forceinline__ void group(int sg, float l, float r, float b, float t) const {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            l = fminf(l, __shfl_xor_sync(kFull, l, o));
            r = fmaxf(r, __shfl_xor_sync(kFull, r, o));
            b = fminf(b, __shfl_xor_sync(kFull, b, o));
            t = fmaxf(t, __shfl_xor_sync(kFull, t, o));
        }
        if ((threadIdx.x & 31) == 0) {
            float4 v = *box;
            if (*seg != sg) {
                if (*seg >= 0) publish(*seg, v);
                v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                *seg = sg;
            }
            *box = make_float4(fminf(v.x, l), fmaxf(v.y, r), fminf(v.z, b), fmaxf(v.w, t));
        }
        __syncwarp();
    }
    // one position written by this lane
    __device__ __forceinline__ void check(float x, float y) const {
        if (!isfinite(x) || !isfinite(y)) atomicOr(status, ST_NONFINITE);
    }
    // whole warp, at its end
    __device__ __forceinline__ void finish() const {
        if ((threadIdx.x & 31) == 0 && *seg >= 0) publish(*seg, *box);
    }
};

// Heaviest groups first.  A group is heavy when the largest previous-step
// group cost carried by its bodies is at least 1.5x its system's mean of the
// previous step (mean > 0): k_frontier lists the heavy groups, and the main
// walk takes them before the others, so that the longest groups do not start
// late and leave the SMs idle.  The largest over the group's bodies, not one
// body's: group boundaries move by a position or two from one step to the
// next, and a group's cost is set mostly by its body of smallest |a| (the
// relative rule), which brings its old group's high cost along when it
// crosses a boundary.  (Plummer 2^20: the first body's cost missed about a
// quarter of the heavy groups, the middle body's an eighth, the largest 4 %.)
struct Heavy {
    const int* list = nullptr;           // heavy group indices, in any order
    const int* count = nullptr;          // their number; null: no reordering
    const int* mean = nullptr;           // [nseg] each system's mean group cost, last step
    unsigned long long* cost = nullptr;  // [nseg] this step's cost (entries x bodies)
};
__device__ __forceinline__ bool heavy_cost(int max_cost, int mean) {
    return mean > 0 && 2ll * max_cost >= 3ll * mean;
}

// Next group for this warp: dynamic scheduling, groups differ ~10x in cost.
__device__ __forceinline__ int next_group(int* work) {
    int g = 0;
    if ((threadIdx.x & 31) == 0) g = atomicAdd(work, 1);
    return __shfl_sync(kFull, g, 0);
}

struct Groups {
    int ngroups;
    const int* gseg_off;  // [nseg+1] first group of each system (nullptr when nseg == 1)
};

__device__ __forceinline__ void group_range(const Segs& segs, const Groups& gr, int g, int* lo,
                                            int* hi, int* gstart, int width = 32,
                                            int* seg = nullptr) {
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
    *gstart = *lo + width * (g - g0);
    if (seg) *seg = s;
}

// ------------------------------------------------------------------ REFERENCE walk

__device__ __forceinline__ float ref_r(float cx, float cy, float px, float py, float eps2, float* dx,
                                       float* dy) {
    *dx = __fsub_rn(cx, px);  // kernels.cu:403-405, no contraction
    *dy = __fsub_rn(cy, py);
    return __fadd_rn(__fadd_rn(__fmul_rn(*dx, *dx), __fmul_rn(*dy, *dy)), eps2);
}

// Rounds of node tests one group may take.  A valid tree gives a group at most
// one test per node, far below this; beyond it the tree is not a tree.
constexpr int kMaxWalkRounds = 1 << 22;

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

// a += m * d * u^-3/2 (softened body-body / monopole term).  With eps2 > 0,
// u > 0 always; with eps2 == 0 the guard drops the self-interaction.
// Potential at p of a cell (monopole + quadrupole about its COM c):
//   phi = -[M u^-1/2 + 0.5 d.T.d u^-5/2 - (h/3) u^-3/2],  d = c - p, T = 3S, h = 1.5 tr S
// (G applied by the caller).
__device__ __forceinline__ float pot_cell(float4 A, float4 B, float px, float py, float eps2) {
    const float dx = A.x - px, dy = A.y - py;
    const float u = fmaf(dx, dx, fmaf(dy, dy, eps2));
    const float ri = rsqrtf(u), r2 = ri * ri, r3 = ri * r2;
    const float tdx = fmaf(B.x, dx, B.y * dy), tdy = fmaf(B.y, dx, B.z * dy);
    const float dtd = fmaf(dx, tdx, dy * tdy);
    return -(A.z * ri + 0.5f * dtd * r3 * r2 - (B.w * (1.0f / 3.0f)) * r3);
}

// PTX rsqrt.approx.ftz.f32: the approximate reciprocal square root without the
// denormal-argument handling that rsqrtf adds (three instructions per call).
// Used where the argument is a squared distance plus a positive softening, or
// a squared distance beyond an opening radius: never a denormal.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// PTX sqrt.approx.ftz.f32 (relative error ~2^-22).  The walk's two rules use
// it with a margin of 2^-18 on the side that opens more nodes, never fewer.
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
constexpr float kRuleMargin = 1.0f - 1.0f / 262144.0f;

template <bool GUARD>
__device__ __forceinline__ void p2p(float bx, float by, float bm, float px, float py, float eps2,
                                    float& ax, float& ay) {
    float dx = bx - px, dy = by - py;
    float u = fmaf(dx, dx, fmaf(dy, dy, eps2));
    float ri = GUARD ? rsqrtf(u) : rsqrt_ftz(u);  // GUARD: eps2 == 0, u may be tiny
    if (GUARD) ri = u > 0.0f ? ri : 0.0f;
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
    float ri = rsqrt_ftz(u);
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

// Two interactions per lane with packed FP32x2 arithmetic (__ffma2_rn and
// friends: per component the same IEEE operations as the scalar code).  The
// walk stages cells and bodies in pairs: component .x belongs to the even
// entry, .y to the odd one.
//   cells:  xy = (x, y)  mh = (M, -h)  t01 = (-T00, -T01)  t11 = -T11   (T = 3S, h = 1.5 tr S)
//   bodies: xy = (x, y)  m              index
// The quadrupole terms are staged negated, so that every subtraction of p2m
// becomes an FMA with a positive addend: -(T d) = T' d, d.T.d = -(d.T'.d).
// Staged cell pairs, one array per component (conflict-free staging stores).
struct CellPairs {
    float4* xy;   // x0 x1 y0 y1
    float4* mh;   // M0 M1 -h0 -h1
    float4* t01;  // -T00_0 -T00_1 -T01_0 -T01_1
    float2* t11;  // -T11_0 -T11_1
};

__device__ __forceinline__ void p2m_pair(const float4 xy, const float4 mh, const float4 t01,
                                         const float2 t11, const float2 npx, const float2 npy,
                                         const float2 e2, float2& ax, float2& ay) {
    const float2 dx = __fadd2_rn(make_float2(xy.x, xy.y), npx);
    const float2 dy = __fadd2_rn(make_float2(xy.z, xy.w), npy);
    const float2 u = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, e2));
    const float2 ri = make_float2(rsqrt_ftz(u.x), rsqrt_ftz(u.y));
    const float2 r2 = __fmul2_rn(ri, ri);
    const float2 r3 = __fmul2_rn(ri, r2);
    const float2 txx = make_float2(t01.x, t01.y), txy = make_float2(t01.z, t01.w);
    const float2 tdx = __ffma2_rn(txx, dx, __fmul2_rn(txy, dy));  // -(T d).x
    const float2 tdy = __ffma2_rn(txy, dx, __fmul2_rn(t11, dy));  // -(T d).y
    const float2 qx = __fmul2_rn(r2, tdx), qy = __fmul2_rn(r2, tdy);  // -(T d) / u
    const float2 w = __ffma2_rn(dx, qx, __fmul2_rn(dy, qy));           // -d.T.d / u
    const float2 t = __ffma2_rn(make_float2(-2.5f, -2.5f), w,
                                make_float2(mh.z, mh.w));              // 2.5 d.T.d / u - h
    const float2 coef = __ffma2_rn(r2, t, make_float2(mh.x, mh.y));
    const float2 fx = __ffma2_rn(coef, dx, qx);
    const float2 fy = __ffma2_rn(coef, dy, qy);
    ax = __ffma2_rn(r3, fx, ax);
    ay = __ffma2_rn(r3, fy, ay);
}

__device__ __forceinline__ void p2p_pair(const float4 xy, const float2 m, const float2 npx,
                                         const float2 npy, const float2 e2, float2& ax,
                                         float2& ay) {
    const float2 dx = __fadd2_rn(make_float2(xy.x, xy.y), npx);
    const float2 dy = __fadd2_rn(make_float2(xy.z, xy.w), npy);
    const float2 u = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, e2));
    const float2 ri = make_float2(rsqrt_ftz(u.x), rsqrt_ftz(u.y));
    const float2 f = __fmul2_rn(__fmul2_rn(m, ri), __fmul2_rn(ri, ri));
    ax = __ffma2_rn(f, dx, ax);
    ay = __ffma2_rn(f, dy, ay);
}

// One staged cell (entry e) back in the record layout of p2m / pot_cell.
__device__ __forceinline__ void unpair_cell(const CellPairs& cp, int e, float4& A, float4& B) {
    const int q = e >> 1;
    const float4 xy = cp.xy[q], mh = cp.mh[q], t01 = cp.t01[q];
    const float2 t11 = cp.t11[q];
    if (e & 1) {
        A = make_float4(xy.y, xy.w, mh.y, 0.0f);
        B = make_float4(-t01.y, -t01.w, -t11.y, -mh.w);
    } else {
        A = make_float4(xy.x, xy.z, mh.x, 0.0f);
        B = make_float4(-t01.x, -t01.z, -t11.x, -mh.z);
    }
}

// Launch-time shape of the accuracy walk (chosen by bh_autotune or the defaults).
struct AccShape {
    int stack;   // stack entries per warp
    int bucket;  // a node of <= bucket bodies is a leaf: its bodies interact directly
    int bpl;     // bodies per lane: a warp walks for a group of 32 * bpl bodies (1 or 2)
};

// Slices a shared walk group lists before its owner adds them up (see the
// shared groups below).
constexpr int kOwnSlices = 64;

// Per-warp shared memory of the accuracy walk (bytes, 16-byte aligned pieces):
// staged cell records and bodies (with 128 spare bytes), a shared group's
// slice list (walks that share groups), the group's positions, the cell list,
// the node stack and the body list.
__host__ __device__ constexpr int acc_body_cap(int bucket) {
    return 32 + 32 * (bucket > 4 ? bucket : 4);
}
__host__ __device__ constexpr int acc_own_bytes(bool share) { return share ? kOwnSlices * 8 : 0; }
__host__ __device__ constexpr int acc_warp_bytes(AccShape sh, bool share = false) {
    return 3 * 32 * 16 + acc_own_bytes(share) + 32 * 8 * sh.bpl + 16 + 64 * 4 +
           ((sh.stack * 4 + 15) & ~15) + ((acc_body_cap(sh.bucket) * 4 + 15) & ~15);
}

// ------------------------------------------------------------------ shared frontier
//
// Consecutive groups open the same nodes near the top of the tree.  For each
// super-group of 2^kSuperLog2 consecutive bodies of one system (counted from
// the system's first body, so a system gets the same frontiers alone and in a
// batch), k_frontier opens once every node that each of its groups would
// open, and keeps the nodes where that stops: the frontier.  The main accuracy
// walk of a group starts from its super-group's frontier instead of the root,
// and tests and decides exactly the nodes it would have tested from the root
// (orc_frontier_check restates this on the CPU).  k_frontier also lists the
// super-group's heavy walk groups (Heavy).
//
// A node is opened for all groups when it is not a leaf bucket, all its
// children are nodes, and the farthest corner of the super-group's box lies
// within its opening radius: far^2 <= ropen^2.  Every distance a group's rule
// can use (box lower bound, extreme-body bound, exact minimum) is a float
// expression of the same form over coordinates inside that box, and is
// monotone in them, so it is <= far^2 and the group does not accept the node.
// A frontier node is accepted by all groups when the super-group box's
// nearest point lies beyond its opening radius and the relative rule holds
// there with the smallest group scale a_g of the super-group (taken 0.1 %
// low, for the groups' own float sums); those cells go to every group's cell
// list untested.  list[S] holds the nodes to test from the front and the
// accepted cells from the back; count[S] = (nodes to test, accepted cells).
//
// The REFERENCE walk (k_walk_vote) starts from frontiers of the reference's
// rule (k_frontier<.., true>): a group opens a cell iff one of its bodies has
// r_b < dp (kernels.cu:395-406), so the cell is opened for all when r of the
// super-group box's corner farthest from the centre of mass is below dp (every
// body's r is at most that: each float step of r is monotone in |dx|, |dy|),
// and approximated by all when dp <= r of the box's nearest point.

constexpr int kSuperLog2 = 9;         // 512 bodies per super-group
constexpr int kFrontierCap = 512;     // frontier entries kept per super-group
constexpr int kFrontierStack = 1024;  // traversal stack per warp of k_frontier

struct Frontier {
    const int* list = nullptr;     // [super-group][kFrontierCap]
    const int2* count = nullptr;   // [super-group]: (nodes to test, accepted cells); x = -1: start
                                   // from the root; null: off
    const int* sup_off = nullptr;  // [nseg+1] first super-group of each system (null: one system)
};

// ------------------------------------------------------------------ REFERENCE walk, batched
//
// k_walk_vote gives the reference's interaction set with the accuracy walk's
// machinery.  The reference approximates a cell iff every lane of the warp
// votes dp_L <= r_b, with r_b = fl(fl(fl(dx)^2 + fl(dy)^2) + eps2) for its
// body b (kernels.cu:395-406): that is, iff dp_L <= min_b r_b.  Lanes test up
// to 32 stack nodes at once and find that minimum as the accuracy walk finds
// its group distance: r of the group box's nearest point is a lower bound
// (every float step is monotone in |dx|, |dy|), r of the four extreme bodies an
// upper bound, and only between the two is the minimum over the bodies taken.
// Accepted cells and the bodies of opened cells are staged and evaluated 32 at
// a time with the reference's arithmetic (kernels.cu:403-411); only the
// summation order differs from the reference.
constexpr int kVoteWarps = 4;
constexpr int kVoteStack = 1024;

// k staged entries (positions xy[e], masses m[e]) added to (ax, ay) in entry
// order with the reference's arithmetic (kernels.cu:403-411): d = c - p,
// r = (dx dx + dy dy) + eps2 uncontracted, f = ((m ri) ri) ri, a += f d.
// Two entries at a time in packed FP32x2 operations, each element rounded as
// the scalar operation is, and one accumulation chain, so the sums are those of
// the scalar loop bit for bit.  FTZ (eps2 a normal float, so r >= eps2 is never
// a denormal): rsqrt.approx.ftz, equal to rsqrtf for every normal argument.
template <bool FTZ>
__device__ __forceinline__ void vote_interact(const float2* __restrict__ xy,
                                              const float* __restrict__ m, int k, float px,
                                              float py, float eps2, float& ax, float& ay) {
    const float2 np = make_float2(-px, -py);
    const float2 e2 = make_float2(eps2, eps2);
    float2 acc = make_float2(ax, ay);
    int e = 0;
    for (; e + 1 < k; e += 2) {
        const float4 c = *reinterpret_cast<const float4*>(xy + e);  // two entries' x, y
        const float2 mm = *reinterpret_cast<const float2*>(m + e);
        const float2 d0 = __fadd2_rn(make_float2(c.x, c.y), np);
        const float2 d1 = __fadd2_rn(make_float2(c.z, c.w), np);
        const float2 q0 = __fmul2_rn(d0, d0), q1 = __fmul2_rn(d1, d1);
        const float2 r = __fadd2_rn(make_float2(__fadd_rn(q0.x, q0.y), __fadd_rn(q1.x, q1.y)), e2);
        const float2 ri = FTZ ? make_float2(rsqrt_ftz(r.x), rsqrt_ftz(r.y))
                              : make_float2(rsqrtf(r.x), rsqrtf(r.y));
        const float2 f = __fmul2_rn(__fmul2_rn(__fmul2_rn(mm, ri), ri), ri);
        acc = __ffma2_rn(make_float2(f.x, f.x), d0, acc);
        acc = __ffma2_rn(make_float2(f.y, f.y), d1, acc);
    }
    if (e < k) {
        const float2 c = xy[e];
        float dx, dy;
        const float r = ref_r(c.x, c.y, px, py, eps2, &dx, &dy);
        const float ri = FTZ ? rsqrt_ftz(r) : rsqrtf(r);
        const float f = m[e] * ri * ri * ri;
        acc = __ffma2_rn(make_float2(f, f), make_float2(dx, dy), acc);
    }
    ax = acc.x;
    ay = acc.y;
}

__device__ __forceinline__ float ref_r_only(float cx, float cy, float px, float py, float eps2) {
    float dx, dy;
    return ref_r(cx, cy, px, py, eps2, &dx, &dy);
}

static __global__ void __launch_bounds__(kVoteWarps * 32) k_walk_vote(Segs segs, Groups gr, WalkIn in,
                                                               const float4* __restrict__ recA,
                                                               const int4* __restrict__ recC,
                                                               float eps2, float dt, float ddt,
                                                               WalkOut out,
                                                               int* __restrict__ status,
                                                               unsigned long long* __restrict__ inter_total,
                                                               int* __restrict__ work,
                                                               Frontier fr) {
    pdl_wait();
    __shared__ int s_stack[kVoteWarps][kVoteStack];
    __shared__ __align__(16) float2 s_sxy[kVoteWarps][32];  // staged entries: x, y
    __shared__ __align__(8) float s_sm[kVoteWarps][32];     // and m
    __shared__ float2 s_gp[kVoteWarps][32];     // the group's positions
    __shared__ int s_clist[kVoteWarps][64];
    __shared__ int s_blist[kVoteWarps][32 + 128];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = lanemask_lt();
    int* stack = s_stack[warp];
    float2* sxy = s_sxy[warp];
    float* smass = s_sm[warp];
    const bool ftz = eps2 >= 0x1p-126f;  // a normal float
    float2* gp = s_gp[warp];
    int* clist = s_clist[warp];
    int* blist = s_blist[warp];
    unsigned long long my_inter = 0;
    __shared__ float4 s_fold[kVoteWarps];
    __shared__ int s_fold_seg[kVoteWarps];
    const BoxFold fold{s_fold + warp, s_fold_seg + warp, out.box_next, status};
    if (out.box_next) fold.init();
    for (int g = next_group(work); g < gr.ngroups; g = next_group(work)) {
        int lo, hi, gstart, sg;
        group_range(segs, gr, g, &lo, &hi, &gstart, 32, &sg);
        const int j = gstart + lane;
        const bool valid = j < hi;
        const int cnt = min(32, hi - gstart);
        // invalid lanes mirror the group's first body (they vote with it)
        const float px = in.x[valid ? j : gstart], py = in.y[valid ? j : gstart];
        __syncwarp();
        gp[lane] = make_float2(px, py);
        float gx0 = px, gx1 = px, gy0 = py, gy1 = py;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            gx0 = fminf(gx0, __shfl_xor_sync(kFull, gx0, o));
            gx1 = fmaxf(gx1, __shfl_xor_sync(kFull, gx1, o));
            gy0 = fminf(gy0, __shfl_xor_sync(kFull, gy0, o));
            gy1 = fmaxf(gy1, __shfl_xor_sync(kFull, gy1, o));
        }
        // the extreme bodies: y at min/max x, x at min/max y
        float ext[4];
        {
            const float key[4] = {gx0, gx1, gy0, gy1};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const unsigned hit = __ballot_sync(kFull, (q < 2 ? px : py) == key[q]);
                ext[q] = __shfl_sync(kFull, q < 2 ? py : px, __ffs(hit) - 1);
            }
        }
        float ax = 0.0f, ay = 0.0f;
        long long entries = 0;
        bool overflow = false;
        int top = 0, ccnt = 0, bcnt = 0, rounds = 0;
        const int* fl = nullptr;  // the super-group's frontier (k_frontier<.., true>), if any
        int nacc = 0;             // its cells that every group approximates
        if (hi - lo >= 2) {
            const int S = (fr.sup_off ? __ldg(fr.sup_off + sg) : 0) + ((gstart - lo) >> kSuperLog2);
            const int2 fc = fr.count ? fr.count[S] : make_int2(-1, 0);
            if (fc.x >= 0 && 2 * fc.x <= kVoteStack) {
                fl = fr.list + (size_t)S * kFrontierCap;
                for (int e = lane; e < fc.x; e += 32) stack[e] = fl[e];
                top = fc.x;
                nacc = fc.y;
            } else {
                if (lane == 0) stack[0] = lo;  // the system's root
                top = 1;
            }
        }
        // k entries of staged (x, y, m), with the reference's arithmetic
        auto interact = [&](int k) {
            if (ftz)
                vote_interact<true>(sxy, smass, k, px, py, eps2, ax, ay);
            else
                vote_interact<false>(sxy, smass, k, px, py, eps2, ax, ay);
            entries += k;
        };
        auto flush_cells = [&](int k) {  // the last k entries of clist
            __syncwarp();
            if (lane < k) {
                const float4 A = recA[kRecStride * (clist[ccnt - k + lane])];
                sxy[lane] = make_float2(A.x, A.y);
                smass[lane] = A.z;
            }
            __syncwarp();
            interact(k);
            ccnt -= k;
        };
        auto flush_bodies = [&](int k) {
            __syncwarp();
            if (lane < k) {
                const int b = blist[bcnt - k + lane];
                sxy[lane] = make_float2(in.x[b], in.y[b]);
                smass[lane] = in.m[b];
            }
            __syncwarp();
            interact(k);
            bcnt -= k;
        };
        // cells every group of the super-group approximates: straight to the cell list
        for (int base = 0; base < nacc; base += 32) {
            const int k = min(32, nacc - base);
            __syncwarp();
            if (lane < k) clist[ccnt + lane] = fl[kFrontierCap - 1 - (base + lane)];
            ccnt += k;
            __syncwarp();
            while (ccnt >= 32) flush_cells(32);
        }
        while (top > 0) {
            if (rounds == kMaxWalkRounds) {  // far beyond any valid tree: report, do not loop
                if (lane == 0) atomicOr(status, ST_TREE);
                break;
            }
            int k = min(32, top);
            if (top + 3 * k > kVoteStack) {  // pop k, push <= 4k
                k = max((kVoteStack - top) / 3, 0);
                if (k == 0) {
                    overflow = true;
                    break;
                }
            }
            __syncwarp();
            const int node = lane < k ? stack[top - 1 - lane] : -1;
            top -= k;
            ++rounds;
            float4 A = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            bool acc = false, need = false;
            if (node >= 0) {
                A = recA[kRecStride * node];
                // lower bound of min_b r_b: the box's nearest point
                const float nx = fminf(fmaxf(A.x, gx0), gx1), ny = fminf(fmaxf(A.y, gy0), gy1);
                const float rlo = ref_r_only(A.x, A.y, nx, ny, eps2);
                if (A.w <= rlo) {
                    acc = true;
                } else {
                    // upper bound: the extreme bodies; below dp some body votes to open
                    float rhi = ref_r_only(A.x, A.y, gx0, ext[0], eps2);
                    rhi = fminf(rhi, ref_r_only(A.x, A.y, gx1, ext[1], eps2));
                    rhi = fminf(rhi, ref_r_only(A.x, A.y, ext[2], gy0, eps2));
                    rhi = fminf(rhi, ref_r_only(A.x, A.y, ext[3], gy1, eps2));
                    need = A.w <= rhi;
                }
            }
            unsigned nm = __ballot_sync(kFull, need);
            while (nm) {  // the exact minimum over the group's bodies, one node at a time
                const int src = __ffs(nm) - 1;
                nm &= nm - 1;
                const float cx = __shfl_sync(kFull, A.x, src), cy = __shfl_sync(kFull, A.y, src);
                float r = ref_r_only(cx, cy, px, py, eps2);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) r = fminf(r, __shfl_xor_sync(kFull, r, o));
                if (lane == src) acc = A.w <= r;
            }
            const unsigned mc = __ballot_sync(kFull, acc);
            if (acc) clist[ccnt + __popc(mc & lt)] = node;
            ccnt += __popc(mc);
            const bool open = node >= 0 && !acc;
            int4 C = make_int4(kNoChild, kNoChild, kNoChild, kNoChild);
            if (open) C = recC[node];
            const int cs[4] = {C.x, C.y, C.z, C.w};
            int nb = 0, nn = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                nb += (cs[q] != kNoChild && cs[q] < 0);
                nn += (cs[q] >= 0);
            }
            int tot;
            const int off = warp_excl_scan(nb | (nn << 16), &tot);
            __syncwarp();  // every lane has read its stack slot before children overwrite it
            if (open) {
                int* bw = blist + bcnt + (off & 0xffff);
                int* nw = stack + top + (off >> 16);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (cs[q] == kNoChild) continue;
                    if (cs[q] < 0)
                        *bw++ = ~cs[q];  // bodies always interact (kernels.cu:395-399)
                    else
                        *nw++ = cs[q];
                }
            }
            bcnt += tot & 0xffff;
            top += tot >> 16;
            __syncwarp();
            while (ccnt >= 32) flush_cells(32);
            while (bcnt >= 32) flush_bodies(32);
        }
        if (ccnt > 0) flush_cells(ccnt);
        if (bcnt > 0) flush_bodies(bcnt);
        if (overflow && lane == 0) atomicOr(status, ST_STACK);
        my_inter += (unsigned long long)(entries * cnt);
        float wl = 0.0f, wr = 0.0f, wb = 0.0f, wt = 0.0f;  // new positions' box, from the origin
        if (valid && !out.x) {
            // forces only (the drop-in's CalculateForces, kernels.cu:340-435): the
            // accelerations in the caller's order, id[] the caller index
            out.ax[in.id[j]] = ax;
            out.ay[in.id[j]] = ay;
        } else if (valid) {
            // kernels.cu:529-533: v += dt*a; x += d*dt*v
            float vx = __fadd_rn(in.vx[j], __fmul_rn(dt, ax));
            float vy = __fadd_rn(in.vy[j], __fmul_rn(dt, ay));
            const float nx = __fadd_rn(px, __fmul_rn(ddt, vx));
            const float ny = __fadd_rn(py, __fmul_rn(ddt, vy));
            fold.check(nx, ny);
            wl = fminf(wl, nx);
            wr = fmaxf(wr, nx);
            wb = fminf(wb, ny);
            wt = fmaxf(wt, ny);
            out.x[j] = nx;
            out.y[j] = ny;
            out.vx[j] = vx;
            out.vy[j] = vy;
            out.m[j] = in.m[j];
            out.id[j] = in.id[j];
            out.ax[j] = ax;
            out.ay[j] = ay;
        }
        if (out.box_next) fold.group(sg, wl, wr, wb, wt);
    }
    if (out.box_next) fold.finish();
    if (lane == 0 && my_inter) atomicAdd(inter_total, my_inter);
}

__host__ __device__ __forceinline__ int num_supers(int n) {
    return (n + (1 << kSuperLog2) - 1) >> kSuperLog2;
}

// One warp per super-group (positions x, y and |a_old| in key order; walk
// records of the systems' trees; sup_off: first super-group of each system,
// null for one; gw: bodies per walk group; alpha: the relative rule's).
template <int WARPS, bool VOTE = false>
__global__ void __launch_bounds__(WARPS * 32) k_frontier(Segs segs, int nsupers,
                                                         const float* __restrict__ x,
                                                         const float* __restrict__ y,
                                                         const float* __restrict__ amag,
                                                         const float4* __restrict__ recA,
                                                         const int4* __restrict__ recC,
                                                         const int4* __restrict__ recD, int bucket,
                                                         int gw, float alpha,
                                                         int* __restrict__ list,
                                                         int2* __restrict__ count,
                                                         const int* __restrict__ sup_off,
                                                         const int* __restrict__ gcost,
                                                         const int* __restrict__ gseg_off,
                                                         const int* __restrict__ mean_cost,
                                                         int* __restrict__ heavy,
                                                         int* __restrict__ nheavy, float eps2) {
    pdl_wait();
    __shared__ int s_stack[WARPS][kFrontierStack];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int S = blockIdx.x * WARPS + warp;
    if (S >= nsupers) return;
    const unsigned lt = lanemask_lt();
    int* stack = s_stack[warp];
    int sg = 0;  // the system: sup_off[sg] <= S < sup_off[sg + 1]
    if (segs.nseg > 1) {
        int a = 0, b = segs.nseg;
        while (b - a > 1) {
            const int mid = (a + b) >> 1;
            if (__ldg(sup_off + mid) <= S)
                a = mid;
            else
                b = mid;
        }
        sg = a;
    }
    const int lo = segs.off[sg], hi = segs.off[sg + 1];
    const int s0 = lo + ((S - (segs.nseg > 1 ? __ldg(sup_off + sg) : 0)) << kSuperLog2);
    const int s1 = min(hi, s0 + (1 << kSuperLog2));
    if (!VOTE) {
        // this super-group's heavy walk groups (at most 32: gw >= 32 bodies).
        // Load k of a lane reads position s0 + 32 k + lane: the 32-body slice
        // k of the super-group, which belongs to group (32 k) / gw.
        constexpr int kSlices = (1 << kSuperLog2) / 32;
        int v[kSlices];
#pragma unroll
        for (int k = 0; k < kSlices; ++k) {
            const int i = s0 + 32 * k + lane;
            v[k] = i < s1 ? __ldg(gcost + i) : 0;
        }
        const int mean = mean_cost[sg];
        const int per = gw >> 5;  // slices per group
        unsigned hm = 0;          // bit q: group q of the super-group is heavy
#pragma unroll
        for (int k = 0; k < kSlices; ++k) {
            int mx = v[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
            if (s0 + 32 * k < s1 && heavy_cost(mx, mean)) hm |= 1u << (k / per);
        }
        int base = 0;
        if (lane == 0 && hm) base = atomicAdd(nheavy, __popc(hm));
        base = __shfl_sync(kFull, base, 0);
        if ((hm >> lane) & 1u)
            heavy[base + __popc(hm & lt)] =
                (segs.nseg > 1 ? __ldg(gseg_off + sg) : 0) + (s0 + lane * gw - lo) / gw;
    }
    float bx0 = __int_as_float(0x7f800000), bx1 = -bx0, by0 = bx0, by1 = -bx0;
    for (int i = s0 + lane; i < s1; i += 32) {
        const float px = x[i], py = y[i];
        bx0 = fminf(bx0, px);
        bx1 = fmaxf(bx1, px);
        by0 = fminf(by0, py);
        by1 = fmaxf(by1, py);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bx0 = fminf(bx0, __shfl_xor_sync(kFull, bx0, o));
        bx1 = fmaxf(bx1, __shfl_xor_sync(kFull, bx1, o));
        by0 = fminf(by0, __shfl_xor_sync(kFull, by0, o));
        by1 = fmaxf(by1, __shfl_xor_sync(kFull, by1, o));
    }
    // the smallest relative-rule scale over the super-group's groups (taken
    // before the traversal, which classifies each frontier node as it stops)
    float aa = __int_as_float(0x7f800000);
    if (!VOTE && alpha > 0.0f) {
        for (int g0 = s0 + lane * gw; g0 < s1; g0 += 32 * gw) {
            const int g1 = min(s1, g0 + gw);
            float amin = __int_as_float(0x7f800000), asum = 0.0f;
            for (int i = g0; i < g1; ++i) {
                const float a = amag[i];
                amin = fminf(amin, a);
                asum += a;
            }
            aa = fminf(aa, alpha * fmaxf(amin, 0.1f * asum / (float)(g1 - g0)));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) aa = fminf(aa, __shfl_xor_sync(kFull, aa, o));
        aa *= 0.999f;
    }
    // The frontier in traversal order, split as it is found: nodes to test from
    // the front of the list, accepted cells from the back.
    int* out = list + (size_t)S * kFrontierCap;
    bool bad = hi - lo < 2;  // no tree: the walk has nothing to start from
    int top = 0, nt = 0, na = 0, rounds = 0;
    if (!bad) {
        if (lane == 0) stack[0] = lo;  // the system's root
        top = 1;
    }
    while (top > 0 && !bad) {
        const int k = min(32, top);
        if (++rounds > kMaxWalkRounds || top + 3 * k > kFrontierStack) {
            bad = true;  // not a valid tree, or too wide a frontier: walks start at the root
            break;
        }
        __syncwarp();
        const int node = lane < k ? stack[top - 1 - lane] : -1;
        top -= k;
        bool open = false, acc = false;
        int4 C = make_int4(kNoChild, kNoChild, kNoChild, kNoChild);
        if (node >= 0) {
            // the children's record with the node's: one L2 round trip per round
            const float4 A = recA[kRecStride * node];
            const int4 D = recD[kRecStride * node];
            const int4 Cn = recC[node];
            bool within;
            if (VOTE) {
                // the reference's rule (kernels.cu:395-406): a group opens the node
                // iff one of its bodies has r < dp; r of the box corner farthest
                // from the centre of mass bounds every body's r from above
                const float fxp =
                    fabsf(__fsub_rn(A.x, bx0)) >= fabsf(__fsub_rn(A.x, bx1)) ? bx0 : bx1;
                const float fyp =
                    fabsf(__fsub_rn(A.y, by0)) >= fabsf(__fsub_rn(A.y, by1)) ? by0 : by1;
                within = ref_r_only(A.x, A.y, fxp, fyp, eps2) < A.w;
            } else {
                const float fx = fmaxf(fabsf(A.x - bx0), fabsf(A.x - bx1));
                const float fy = fmaxf(fabsf(A.y - by0), fabsf(A.y - by1));
                within = fmaf(fx, fx, fy * fy) <= A.w;
            }
            if (D.y > bucket && within) {
                C = Cn;
                open = (C.x >= 0 || C.x == kNoChild) && (C.y >= 0 || C.y == kNoChild) &&
                       (C.z >= 0 || C.z == kNoChild) && (C.w >= 0 || C.w == kNoChild);
            }
            if (!open && VOTE) {
                // every group approximates it: dp <= r of the box's nearest point
                const float nx = fminf(fmaxf(A.x, bx0), bx1), ny = fminf(fmaxf(A.y, by0), by1);
                acc = A.w <= ref_r_only(A.x, A.y, nx, ny, eps2);
            } else if (!open) {
                // a frontier node: accepted by every group of the super-group
                // when its box's nearest point is beyond the opening radius and
                // the relative rule holds there at the smallest group scale
                const float ddx = fmaxf(fmaxf(bx0 - A.x, A.x - bx1), 0.0f);
                const float ddy = fmaxf(fmaxf(by0 - A.y, A.y - by1), 0.0f);
                const float d2 = fmaf(ddx, ddx, ddy * ddy);
                if (d2 > A.w)
                    acc = __int_as_float(D.z) <= aa * kRuleMargin * d2 * d2 * sqrt_approx(d2);
            }
        }
        const int nn = open ? (C.x >= 0) + (C.y >= 0) + (C.z >= 0) + (C.w >= 0) : 0;
        const unsigned am = __ballot_sync(kFull, node >= 0 && !open && acc);
        const unsigned tm = __ballot_sync(kFull, node >= 0 && !open && !acc);
        int ntot;
        const int noff = warp_excl_scan(nn, &ntot);
        __syncwarp();  // every lane has read its stack slot before children overwrite it
        if (open) {
            int* w = stack + top + noff;
            if (C.x >= 0) *w++ = C.x;
            if (C.y >= 0) *w++ = C.y;
            if (C.z >= 0) *w++ = C.z;
            if (C.w >= 0) *w++ = C.w;
        }
        if (node >= 0 && !open) {
            // in bounds whatever the count; a list over kFrontierCap is discarded
            if (acc) {
                const int idx = na + __popc(am & lt);
                if (idx < kFrontierCap) out[kFrontierCap - 1 - idx] = node;
            } else {
                const int idx = nt + __popc(tm & lt);
                if (idx < kFrontierCap) out[idx] = node;
            }
        }
        top += ntot;
        nt += __popc(tm);
        na += __popc(am);
    }
    if (lane == 0) count[S] = (bad || nt + na > kFrontierCap) ? make_int2(-1, 0) : make_int2(nt, na);
}

// Below this many lanes the exact group distance is taken cooperatively
// (each lane measures its own body, then a warp minimum) instead of by a
// loop over the 32 bodies in every lane.
constexpr int kSerialExactLanes = 8;

// The sum of one staged batch for each of a lane's bodies: the value the walk
// adds to its running sums.  k cells as quadrupoles (cells_sum) or k bodies
// (bodies_sum), pairs in FP32x2 and an odd last entry in scalar arithmetic.
// The walk's own batches and the batches of a shared group evaluated by
// another warp both go through these, so a batch sums to the same floats
// whichever warp evaluates it.
template <int BPL>
__device__ __forceinline__ void cells_sum(const CellPairs& cp, int k, const float (&px)[BPL],
                                          const float (&py)[BPL], const float2 (&npx)[BPL],
                                          const float2 (&npy)[BPL], float eps2, float (&ox)[BPL],
                                          float (&oy)[BPL]) {
    const float2 e2v = make_float2(eps2, eps2);
    float bx[BPL], by[BPL];
    float2 sx[BPL], sy[BPL];
#pragma unroll
    for (int b = 0; b < BPL; ++b) {
        bx[b] = by[b] = 0.0f;
        sx[b] = sy[b] = make_float2(0.0f, 0.0f);
    }
    if (k == 32) {
#pragma unroll 8
        for (int e = 0; e < 16; ++e) {
            const float4 xy = cp.xy[e], mh = cp.mh[e], t01 = cp.t01[e];
            const float2 t11 = cp.t11[e];
#pragma unroll
            for (int b = 0; b < BPL; ++b) p2m_pair(xy, mh, t01, t11, npx[b], npy[b], e2v, sx[b], sy[b]);
        }
    } else {
        for (int e = 0; e < (k >> 1); ++e) {
            const float4 xy = cp.xy[e], mh = cp.mh[e], t01 = cp.t01[e];
            const float2 t11 = cp.t11[e];
#pragma unroll
            for (int b = 0; b < BPL; ++b) p2m_pair(xy, mh, t01, t11, npx[b], npy[b], e2v, sx[b], sy[b]);
        }
        if (k & 1) {
            float4 A, B;
            unpair_cell(cp, k - 1, A, B);
#pragma unroll
            for (int b = 0; b < BPL; ++b) p2m(A, B, px[b], py[b], eps2, bx[b], by[b]);
        }
    }
#pragma unroll
    for (int b = 0; b < BPL; ++b) {
        ox[b] = bx[b] + (sx[b].x + sx[b].y);
        oy[b] = by[b] + (sy[b].x + sy[b].y);
    }
}

template <int BPL>
__device__ __forceinline__ void bodies_sum(const float4* bxy, const float2* bm, int k,
                                           const float (&px)[BPL], const float (&py)[BPL],
                                           const float2 (&npx)[BPL], const float2 (&npy)[BPL],
                                           float eps2, float (&ox)[BPL], float (&oy)[BPL]) {
    const float2 e2v = make_float2(eps2, eps2);
    // entry e of the staged bodies, unpaired
    auto body = [&](int e, float& x, float& y, float& m) {
        const float4 q = bxy[e >> 1];
        const float2 w = bm[e >> 1];
        x = (e & 1) ? q.y : q.x;
        y = (e & 1) ? q.w : q.z;
        m = (e & 1) ? w.y : w.x;
    };
    float bx[BPL], by[BPL];
    float2 sx[BPL], sy[BPL];
#pragma unroll
    for (int b = 0; b < BPL; ++b) {
        bx[b] = by[b] = 0.0f;
        sx[b] = sy[b] = make_float2(0.0f, 0.0f);
    }
    if (eps2 > 0.0f) {
        if (k == 32) {
#pragma unroll 8
            for (int e = 0; e < 16; ++e) {
                const float4 xy = bxy[e];
                const float2 w = bm[e];
#pragma unroll
                for (int b = 0; b < BPL; ++b) p2p_pair(xy, w, npx[b], npy[b], e2v, sx[b], sy[b]);
            }
        } else {
            for (int e = 0; e < (k >> 1); ++e) {
                const float4 xy = bxy[e];
                const float2 w = bm[e];
#pragma unroll
                for (int b = 0; b < BPL; ++b) p2p_pair(xy, w, npx[b], npy[b], e2v, sx[b], sy[b]);
            }
            if (k & 1) {
                float x, y, m;
                body(k - 1, x, y, m);
#pragma unroll
                for (int b = 0; b < BPL; ++b) p2p<false>(x, y, m, px[b], py[b], eps2, bx[b], by[b]);
            }
        }
    } else {
        for (int e = 0; e < k; ++e) {
            float x, y, m;
            body(e, x, y, m);
#pragma unroll
            for (int b = 0; b < BPL; ++b) p2p<true>(x, y, m, px[b], py[b], eps2, bx[b], by[b]);
        }
    }
#pragma unroll
    for (int b = 0; b < BPL; ++b) {
        ox[b] = bx[b] + (sx[b].x + sx[b].y);
        oy[b] = by[b] + (sy[b].x + sy[b].y);
    }
}

// ------------------------------------------------------------------ shared groups
//
// The heaviest groups of the main accuracy walk (taken first, they still last
// about as long as the whole walk) keep one warp busy each.  The warp that
// takes a shared group walks the tree for it as usual, but records each batch
// of up to 32 entries it would evaluate (the nodes or the bodies) in a pool
// instead of evaluating it, and publishes the batches kSliceBatches at a time
// as a slice.  A warp between two groups takes a published slice first: it
// evaluates the slice's batches for the group's bodies and stores every
// lane's batch sums.  At the end of its walk the owner evaluates every slice
// that no other warp has taken (the latest first), then adds all batch sums
// in the order it recorded them.  The batch sums are the ones the owner would
// have formed (the same entries, staged the same way, cells_sum / bodies_sum),
// added in the same order: a shared group's results are bit for bit those of
// an unshared one, whichever warps evaluated its batches.  A group that runs
// out of pool or slice list is walked again, unshared.  Every wait is
// bounded: a slice reserved but not yet published is left to its owner, and a
// taken slice that is never finished (a running warp always finishes it) is
// reported as ST_TREE.
// Measured on GB300 (Plummer, MIXED, graph step): sharing the heavy groups
// gains 6 % at 2^16 bodies and 4 % at 2^17, where a system has fewer walk
// groups than the GPU has resident warps, and loses 3-12 % from 2^18 on, where
// every warp has several groups and the pool's extra loads and stores cost
// more than the heavy groups' tail; the host shares by default only below
// that size.
constexpr int kSliceBatches = 8;      // batches per slice (at most 15: 4 bits in the slice list)
constexpr int kReadyPolls = 64;       // polls for a reserved slice to be published
constexpr int kDonePolls = 1 << 18;   // polls for a taken slice to be evaluated (~0.2 s)
// Counters of the shared groups (Share::ctr), each on its own 128-byte line:
// every warp reads the queue's head and tail between groups.
enum : int { kCtrHead = 0, kCtrTail = 1, kCtrBatches = 32, kCtrBack = 64, kCtrWords = 96 };
static_assert(kSliceBatches < 16, "slice list packs the batch count in 4 bits");
enum : int { SL_EMPTY = 0, SL_READY = 1, SL_TAKEN = 2, SL_DONE = 3 };

struct Share {
    int* ctr = nullptr;     // [kCtrWords]: slices handed out (kCtrHead), slices reserved
                            // (kCtrTail), pool batches reserved, slices taken back by their
                            // owners; cleared every step.  null: no sharing
    int* state = nullptr;   // [cap_slices] SL_*, cleared every step
    int4* desc = nullptr;   // [cap_slices] (first batch, batches, group's first body, system end)
    int* idx = nullptr;     // [cap_batches][32] an entry's node, or ~body; INT_MIN past the end
    float2* sum = nullptr;  // [cap_batches][bodies per lane][32] each lane's batch sum (x, y)
    int cap_batches = 0, cap_slices = 0;
    int tail = 0;           // the last `tail` groups handed out are shared as well
};

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_gpu(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// The first value >= least that *p holds, or the last one read after `polls` more reads.
__device__ __forceinline__ int wait_state(const int* p, int least, int polls) {
    int v = ld_acquire_gpu(p);
    for (int i = 0; v < least && i < polls; ++i) {
        __nanosleep(64);
        v = ld_acquire_gpu(p);
    }
    return v;
}
// lane 0: the oldest published slice not yet handed out, now taken by this
// warp (SL_READY -> SL_TAKEN), or -1.  The queue's head moves by atomicAdd (a
// compare-and-swap loop serialises thousands of warps); a warp that moves it
// past the tail in a race, or finds its slice unpublished after kReadyPolls
// reads or taken back by its owner, goes on to the next one.  A slice skipped
// that way is evaluated by its owner.
__device__ __forceinline__ int take_slice(const Share& sh) {
    for (;;) {
        if (ld_relaxed_gpu(sh.ctr + kCtrHead) >= ld_relaxed_gpu(sh.ctr + kCtrTail)) return -1;
        const int s = atomicAdd(sh.ctr + kCtrHead, 1);
        if (s >= sh.cap_slices) return -1;
        if (wait_state(sh.state + s, SL_READY, kReadyPolls) == SL_READY &&
            atomicCAS(sh.state + s, SL_READY, SL_TAKEN) == SL_READY)
            return s;
    }
}

// A warp's staging area at the start of its shared memory: 16 cell pairs
// (896 bytes), 16 body pairs (256 + 128), their indices (128), 128 spare.
__device__ __forceinline__ void acc_staging(unsigned char* wbase, CellPairs& cp, float4*& bxy,
                                            float2*& bm, int2*& bid) {
    cp.xy = reinterpret_cast<float4*>(wbase);
    cp.mh = cp.xy + 16;
    cp.t01 = cp.mh + 16;
    cp.t11 = reinterpret_cast<float2*>(cp.t01 + 16);
    bxy = reinterpret_cast<float4*>(cp.t11 + 16);
    bm = reinterpret_cast<float2*>(bxy + 16);
    bid = reinterpret_cast<int2*>(bm + 16);
}

// Batches first .. first + nb - 1 of the pool (idx) for a group whose lane
// bodies are at (px, py), staged in the warp's staging area (wbase): every
// lane's batch sums to sum[].
template <int BPL>
__device__ __forceinline__ void eval_batches(unsigned char* wbase, const float4* __restrict__ recA,
                                             const float4* __restrict__ recB,
                                             const float* __restrict__ x,
                                             const float* __restrict__ y,
                                             const float* __restrict__ m, const int* idx,
                                             float2* sum, float eps2, int first, int nb,
                                             const float (&px)[BPL], const float (&py)[BPL]) {
    const int lane = threadIdx.x & 31;
    CellPairs cp;
    float4* bxy;
    float2* bm;
    int2* bid;
    acc_staging(wbase, cp, bxy, bm, bid);
    float2 npx[BPL], npy[BPL];
#pragma unroll
    for (int b = 0; b < BPL; ++b) {
        npx[b] = make_float2(-px[b], -px[b]);
        npy[b] = make_float2(-py[b], -py[b]);
    }
    // each batch's entries are loaded one batch ahead
    int vnext = __ldcg(idx + (size_t)first * 32 + lane);
    for (int t = 0; t < nb; ++t) {
        const size_t bt = (size_t)first + t;
        const int v = vnext;
        if (t + 1 < nb) vnext = __ldcg(idx + (bt + 1) * 32 + lane);
        const int k = __popc(__ballot_sync(kFull, v != INT_MIN));  // the entries are a prefix
        const bool body = __shfl_sync(kFull, v, 0) < 0;
        float ox[BPL], oy[BPL];
        __syncwarp();  // the staging area of the last batch is read
        const int q = lane >> 1, h = lane & 1;
        if (body) {
            if (lane < k) {
                const int bi = ~v;
                reinterpret_cast<float*>(&bxy[q])[h] = x[bi];
                reinterpret_cast<float*>(&bxy[q])[2 + h] = y[bi];
                reinterpret_cast<float*>(&bm[q])[h] = m[bi];
            }
            __syncwarp();
            bodies_sum<BPL>(bxy, bm, k, px, py, npx, npy, eps2, ox, oy);
        } else {
            if (lane < k) {
                const float4 A = recA[kRecStride * v], B = recB[v];
                reinterpret_cast<float*>(cp.xy + q)[h] = A.x;
                reinterpret_cast<float*>(cp.xy + q)[2 + h] = A.y;
                reinterpret_cast<float*>(cp.mh + q)[h] = A.z;
                reinterpret_cast<float*>(cp.mh + q)[2 + h] = -B.w;
                reinterpret_cast<float*>(cp.t01 + q)[h] = -B.x;
                reinterpret_cast<float*>(cp.t01 + q)[2 + h] = -B.y;
                reinterpret_cast<float*>(cp.t11 + q)[h] = -B.z;
            }
            __syncwarp();
            cells_sum<BPL>(cp, k, px, py, npx, npy, eps2, ox, oy);
        }
#pragma unroll
        for (int b = 0; b < BPL; ++b)
            __stcg(sum + (bt * BPL + b) * 32 + lane, make_float2(ox[b], oy[b]));
    }
    __syncwarp();
}

// PLAIN / MIXED walk.  ESTIMATE = the bootstrap pass after bh_set_state: the
// geometric rule only, at opening angle max(theta, kBootstrapTheta) (radius
// in recD.w), cells as monopoles, launched with 64-body groups; writes |G a|
// into in.amag and nothing else (skipped unless *fresh is set).  The main pass also applies the relative rule
//   G M l^3 <= alpha * a_g * d^5,  a_g = max(min |a_old|, 0.1 mean |a_old|) over the group,
// d = min over the group's bodies of |COM - p|; the geometric rule is d > l/theta + delta.
// DIAG = diagnostics pass: the main rule, but each body's potential (FP64
// accumulation of float batches, own body excluded) goes to pot[] and nothing
// is integrated.  SHARE = the main pass with shared groups (sh); without it
// none of their code or shared memory is compiled in.
template <bool MIXED, bool ESTIMATE, bool DIAG = false, int BPL = 1, bool SHARE = false>
__global__ void __launch_bounds__(256, BPL == 1 ? 4 : 3) k_walk_acc(AccShape shape, Segs segs, Groups gr, WalkIn in,
                                                         const float4* __restrict__ recA,
                                                         const float4* __restrict__ recB,
                                                         const int4* __restrict__ recC,
                                                         const int4* __restrict__ recD, float eps2,
                                                         float G, float dt, float ddt, float alpha,
                                                         WalkOut out, int* __restrict__ status,
                                                         unsigned long long* __restrict__ inter_total,
                                                         int* __restrict__ work,
                                                         int* __restrict__ fresh,
                                                         int* __restrict__ max_stack,
                                                         double* __restrict__ pot,
                                                         Frontier fr, Heavy hv, Share sh) {
    pdl_wait();
    static_assert(BPL == 1 || BPL == 2, "one or two bodies per lane");
    if (ESTIMATE) {
        if (*(volatile int*)fresh == 0) return;
    } else if (!DIAG && blockIdx.x == 0 && threadIdx.x == 0) {
        *fresh = 0;  // the bootstrap pass of this step (if any) has completed
    }
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = lanemask_lt();
    const int STACK = shape.stack, BUCKET = shape.bucket;
    constexpr int GW = 32 * BPL;  // bodies per group
    unsigned char* wbase = smem_raw + (size_t)warp * acc_warp_bytes(shape, SHARE);
    // 1536 bytes: 16 cell pairs (896), 16 body pairs (512), 128 spare
    CellPairs cpair;
    float4* bxy;
    float2* bm;
    int2* bid;
    acc_staging(wbase, cpair, bxy, bm, bid);
    // the group's GW positions in pairs: (x_2i, x_2i+1, y_2i, y_2i+1)
    float4* gp = reinterpret_cast<float4*>(wbase + 3 * 32 * 16 + acc_own_bytes(SHARE));
    float4* gext = gp + GW / 2;  // y at min/max x, x at min/max y
    int* clist = reinterpret_cast<int*>(gext + 1);
    int* stack = clist + 64;
    int* blist = stack + ((STACK + 3) & ~3);
    unsigned long long my_inter = 0, my_cinter = 0;
    // main pass only (the bootstrap and diagnostics passes write no positions);
    // its shared box sits in the spare bytes after the staged body pairs
    const bool folding = !ESTIMATE && !DIAG && out.box_next != nullptr;
    const BoxFold fold{reinterpret_cast<float4*>(wbase + 1408), reinterpret_cast<int*>(wbase + 1424),
                       out.box_next, status};
    if (folding) fold.init();
    // shared groups (main pass only): this warp's slice list; its open slice
    // as (first batch, batches recorded, slices listed, 1: out of room); its
    // group as (first body, system end, hand-out index, 1: shared)
    const bool sharing = SHARE && !ESTIMATE && !DIAG && sh.ctr != nullptr;
    // (all at fixed offsets: the slice list after the staging area, the rest
    // in its spare bytes after the folded box)
    int2* own = reinterpret_cast<int2*>(wbase + 3 * 32 * 16);
    int4* ows = reinterpret_cast<int4*>(wbase + 1440);
    int4* ogr = reinterpret_cast<int4*>(wbase + 1456);

    // heavy groups first (hv.count set: the main pass), then the others in order
    const int nh = hv.count ? *hv.count : 0;
    const int total = nh + gr.ngroups;
    int retry = -1;  // a shared group that ran out of room, to be walked again unshared
    for (;;) {
        const bool again = retry >= 0;
        int c = retry;
        retry = -1;
        if (!again) {
        if (sharing) {
            // a published slice of a shared group comes before a new group
            int sl = lane == 0 ? take_slice(sh) : -1;
            sl = __shfl_sync(kFull, sl, 0);
            if (sl >= 0) {
                // the slice's group: its first body and its system's end; lanes
                // past the end mirror the first body, as in the walk
                const int4 d = __ldcg(sh.desc + sl);
                float qx[BPL], qy[BPL];
#pragma unroll
                for (int b = 0; b < BPL; ++b) {
                    const int jb = d.z + 32 * b + lane;
                    qx[b] = in.x[jb < d.w ? jb : d.z];
                    qy[b] = in.y[jb < d.w ? jb : d.z];
                }
                eval_batches<BPL>(wbase, recA, recB, in.x, in.y, in.m, sh.idx, sh.sum, eps2, d.x, d.y,
                                  qx, qy);
                __threadfence();  // this lane's sums before the slice is marked done
                __syncwarp();
                if (lane == 0) st_release_gpu(sh.state + sl, SL_DONE);
                continue;
            }
        }
        // (a warp without groups leaves: the owners take back what is left)
        c = next_group(work);
        if (c >= total) break;
        }
        const int g = c < nh ? hv.list[c] : c - nh;
        int lo, hi, gstart, sg;
        group_range(segs, gr, g, &lo, &hi, &gstart, GW, &sg);
        if (c >= nh && nh > 0) {
            // a heavy group was taken first: the same test as k_frontier's
            int mx = 0;
#pragma unroll
            for (int b = 0; b < BPL; ++b)
                if (gstart + 32 * b + lane < hi) mx = max(mx, __ldg(in.gcost + gstart + 32 * b + lane));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
            if (heavy_cost(mx, hv.mean[sg])) continue;  // done first
        }
        const int cnt = min(GW, hi - gstart);
        // body b of this lane is position gstart + 32 b + lane; invalid ones
        // mirror the group's first body
        int j[BPL];
        bool valid[BPL];
        float px[BPL], py[BPL];
#pragma unroll
        for (int b = 0; b < BPL; ++b) {
            j[b] = gstart + 32 * b + lane;
            valid[b] = j[b] < hi;
            const int jj = valid[b] ? j[b] : gstart;
            px[b] = in.x[jj];
            py[b] = in.y[jj];
        }
        __syncwarp();
        float gx0 = px[0], gx1 = px[0], gy0 = py[0], gy1 = py[0];
#pragma unroll
        for (int b = 0; b < BPL; ++b) {
            float* gq = reinterpret_cast<float*>(gp + ((32 * b + lane) >> 1));
            gq[lane & 1] = px[b];
            gq[2 + (lane & 1)] = py[b];
            gx0 = fminf(gx0, px[b]);
            gx1 = fmaxf(gx1, px[b]);
            gy0 = fminf(gy0, py[b]);
            gy1 = fmaxf(gy1, py[b]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            gx0 = fminf(gx0, __shfl_xor_sync(kFull, gx0, o));
            gx1 = fmaxf(gx1, __shfl_xor_sync(kFull, gx1, o));
            gy0 = fminf(gy0, __shfl_xor_sync(kFull, gy0, o));
            gy1 = fmaxf(gy1, __shfl_xor_sync(kFull, gy1, o));
        }
        const float gdiag = sqrtf((gx1 - gx0) * (gx1 - gx0) + (gy1 - gy0) * (gy1 - gy0));
        {
            // the group's extreme bodies in x and y: the nearest of them bounds
            // the exact group distance from above
            float ext[4];
            const float key[4] = {gx0, gx1, gy0, gy1};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float v = 0.0f;
                bool found = false;
#pragma unroll
                for (int b = 0; b < BPL; ++b) {
                    const float c = q < 2 ? px[b] : py[b];
                    const float other = q < 2 ? py[b] : px[b];
                    const unsigned hit = __ballot_sync(kFull, c == key[q]);
                    const float w = __shfl_sync(kFull, other, __ffs(hit) - 1);
                    if (!found && hit) {
                        v = w;
                        found = true;
                    }
                }
                ext[q] = v;
            }
            if (lane == 0) *gext = make_float4(ext[0], ext[1], ext[2], ext[3]);
        }
        // relative-rule scale of the group
        float aa = __int_as_float(0x7f800000);
        if (!ESTIMATE && !DIAG && alpha > 0.0f) {
            float amin = __int_as_float(0x7f800000), asum = 0.0f;
#pragma unroll
            for (int b = 0; b < BPL; ++b) {
                const float a = in.amag[valid[b] ? j[b] : gstart];
                amin = fminf(amin, a);
                asum += valid[b] ? a : 0.0f;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                amin = fminf(amin, __shfl_xor_sync(kFull, amin, o));
                asum += __shfl_xor_sync(kFull, asum, o);
            }
            aa = alpha * fmaxf(amin, 0.1f * asum / (float)cnt);
        }
        if (sharing) {
            // a heavy group, or one of the last `tail` handed out: shared
            // (unless it ran out of room in the pool before)
            const bool shared = !again && (c < nh || c >= total - sh.tail);
            if (lane == 0) {
                *ows = make_int4(0, 0, 0, 0);
                *ogr = make_int4(gstart, hi, c, shared ? 1 : 0);
            }
            __syncwarp();
        }
        float ax[BPL], ay[BPL];    // running sums
        float cax[BPL], cay[BPL];  // Kahan compensation (MIXED)
        double phi[BPL];           // DIAG: potential
#pragma unroll
        for (int b = 0; b < BPL; ++b) ax[b] = ay[b] = cax[b] = cay[b] = 0.0f, phi[b] = 0.0;
        long long entries = 0, centries = 0;
        bool overflow = false;
        int top = 0, ccnt = 0, bcnt = 0, peak = 0, rounds = 0, tested = 0;
        const int* fl = nullptr;  // the super-group's frontier, if the walk starts there
        int nacc = 0;             // its cells that every group accepts
        if (hi - lo >= 2) {
            // the super-group's frontier (main pass), else the root
            const int S = (fr.sup_off ? __ldg(fr.sup_off + sg) : 0) + ((gstart - lo) >> kSuperLog2);
            const int2 fc = fr.count ? fr.count[S] : make_int2(-1, 0);
            if (fc.x >= 0 && 2 * fc.x <= STACK) {
                fl = fr.list + (size_t)S * kFrontierCap;
                for (int e = lane; e < fc.x; e += 32) stack[e] = fl[e];
                top = fc.x;
                nacc = fc.y;
            } else {
                if (lane == 0) stack[0] = lo;
                top = 1;
            }
        }
        auto add_batch = [&](int b, float bx, float by) {
            if (MIXED) {
                float yx = bx - cax[b], tx = ax[b] + yx;
                cax[b] = (tx - ax[b]) - yx;
                ax[b] = tx;
                float yy = by - cay[b], ty = ay[b] + yy;
                cay[b] = (ty - ay[b]) - yy;
                ay[b] = ty;
            } else {
                ax[b] += bx;
                ay[b] += by;
            }
        };
        // packed-pair constants of this lane's bodies
        float2 npx[BPL], npy[BPL];
#pragma unroll
        for (int b = 0; b < BPL; ++b) {
            npx[b] = make_float2(-px[b], -px[b]);
            npy[b] = make_float2(-py[b], -py[b]);
        }
        const float2 e2v = make_float2(eps2, eps2);
        // Shared group: add up the recorded batches, in order.  First every
        // slice that no other warp has taken (the open one, never published,
        // among them) is evaluated here, the latest first, while the others
        // finish theirs; then all batch sums are added in the recorded order,
        // waiting for the slices still being evaluated elsewhere.
        auto combine = [&]() {
            int4 w = *ows;
            __syncwarp();
            if (w.y > 0) {
                if (lane == 0) own[w.z] = make_int2(w.x * 16 + w.y, -1);
                ++w.z;
                __syncwarp();
            }
            for (int i = w.z - 1; i >= 0; --i) {
                const int2 o = own[i];
                int mine = o.y < 0;
                if (!mine && lane == 0 && atomicCAS(sh.state + o.y, SL_READY, SL_TAKEN) == SL_READY) {
                    mine = 1;
                    atomicAdd(sh.ctr + kCtrBack, 1);
                }
                mine = __shfl_sync(kFull, mine, 0);
                if (mine) {
                    eval_batches<BPL>(wbase, recA, recB, in.x, in.y, in.m, sh.idx, sh.sum, eps2,
                                      o.x >> 4, o.x & 15, px, py);
                    if (lane == 0) own[i].y = -1;  // evaluated here: nothing to wait for
                }
            }
            __syncwarp();
            for (int i = 0; i < w.z; ++i) {
                const int2 o = own[i];
                const int first = o.x >> 4, nb = o.x & 15;
                if (o.y >= 0 && lane == 0 && wait_state(sh.state + o.y, SL_DONE, kDonePolls) != SL_DONE)
                    atomicOr(status, ST_TREE);  // never finished: not a running warp's
                __syncwarp();
                for (int t = 0; t < nb; ++t) {
#pragma unroll
                    for (int b = 0; b < BPL; ++b) {
                        const float2 v = __ldcg(sh.sum + ((size_t)(first + t) * BPL + b) * 32 + lane);
                        add_batch(b, v.x, v.y);
                    }
                }
            }
            if (lane == 0) *ows = make_int4(0, 0, 0, 0);
            __syncwarp();
        };
        // Shared group: src[0..k) (nodes, or bodies when `body`) becomes the
        // next recorded batch.  No room in the pool or the slice list: redo.
        auto record = [&](const int* src, int k, bool body) {
            int4 w = *ows;
            __syncwarp();
            if (w.y == 0) {
                int base = INT_MAX;
                if (lane == 0 && w.z < kOwnSlices) base = atomicAdd(sh.ctr + kCtrBatches, kSliceBatches);
                base = __shfl_sync(kFull, base, 0);
                if (base > sh.cap_batches - kSliceBatches) {
                    if (lane == 0) ows->w = 1;  // redo
                    __syncwarp();
                    return;
                }
                w.x = base;
            }
            const int v = lane < k ? (body ? ~src[lane] : src[lane]) : INT_MIN;
            __stcg(sh.idx + (size_t)(w.x + w.y) * 32 + lane, v);
            if (++w.y == kSliceBatches) {
                // publish the slice (or keep it, when the state array is full)
                __threadfence();  // this lane's entries before the slice is published
                __syncwarp();
                if (lane == 0) {
                    int sl = atomicAdd(sh.ctr + kCtrTail, 1);
                    if (sl < sh.cap_slices) {
                        sh.desc[sl] = make_int4(w.x, w.y, ogr->x, ogr->y);
                        st_release_gpu(sh.state + sl, SL_READY);
                    } else {
                        sl = -1;
                    }
                    own[w.z] = make_int2(w.x * 16 + w.y, sl);
                }
                ++w.z;
                w.y = 0;
            }
            if (lane == 0) *ows = w;
            __syncwarp();
        };
        auto flush_cells = [&](int k) {  // the last k entries of clist
            if (sharing && ogr->w) {
                if (!ows->w) record(clist + ccnt - k, k, false);
                ccnt -= k;
                entries += k;
                centries += k;
                return;
            }
            __syncwarp();
            if (lane < k) {
                const int node = clist[ccnt - k + lane];
                const float4 A = recA[kRecStride * node], B = recB[node];
                const int q = lane >> 1, h = lane & 1;
                reinterpret_cast<float*>(cpair.xy + q)[h] = A.x;
                reinterpret_cast<float*>(cpair.xy + q)[2 + h] = A.y;
                reinterpret_cast<float*>(cpair.mh + q)[h] = A.z;
                reinterpret_cast<float*>(cpair.mh + q)[2 + h] = -B.w;
                reinterpret_cast<float*>(cpair.t01 + q)[h] = -B.x;
                reinterpret_cast<float*>(cpair.t01 + q)[2 + h] = -B.y;
                reinterpret_cast<float*>(cpair.t11 + q)[h] = -B.z;
            }
            __syncwarp();
            if (DIAG) {
                float f[BPL];
#pragma unroll
                for (int b = 0; b < BPL; ++b) f[b] = 0.0f;
                for (int e = 0; e < k; ++e) {
                    float4 A, B;
                    unpair_cell(cpair, e, A, B);
#pragma unroll
                    for (int b = 0; b < BPL; ++b) f[b] += pot_cell(A, B, px[b], py[b], eps2);
                }
#pragma unroll
                for (int b = 0; b < BPL; ++b) phi[b] += (double)f[b];
            } else if (ESTIMATE) {
                // the bootstrap needs |a| to a few per cent: monopoles suffice
                float bx[BPL], by[BPL];
                float2 sx[BPL], sy[BPL];
#pragma unroll
                for (int b = 0; b < BPL; ++b) {
                    bx[b] = by[b] = 0.0f;
                    sx[b] = sy[b] = make_float2(0.0f, 0.0f);
                }
                for (int e = 0; e < (k >> 1); ++e) {
                    const float4 mh = cpair.mh[e];
                    const float4 xy = cpair.xy[e];
#pragma unroll
                    for (int b = 0; b < BPL; ++b)
                        p2p_pair(xy, make_float2(mh.x, mh.y), npx[b], npy[b], e2v, sx[b], sy[b]);
                }
                if (k & 1) {
                    float4 A, B;
                    unpair_cell(cpair, k - 1, A, B);
#pragma unroll
                    for (int b = 0; b < BPL; ++b)
                        p2p<false>(A.x, A.y, A.z, px[b], py[b], eps2, bx[b], by[b]);
                }
#pragma unroll
                for (int b = 0; b < BPL; ++b)
                    add_batch(b, bx[b] + (sx[b].x + sx[b].y), by[b] + (sy[b].x + sy[b].y));
            } else {
                float ox[BPL], oy[BPL];
                cells_sum<BPL>(cpair, k, px, py, npx, npy, eps2, ox, oy);
#pragma unroll
                for (int b = 0; b < BPL; ++b) add_batch(b, ox[b], oy[b]);
            }
            ccnt -= k;
            entries += k;
            centries += k;
        };
        auto flush_bodies = [&](int k) {
            if (sharing && ogr->w) {
                if (!ows->w) record(blist + bcnt - k, k, true);
                bcnt -= k;
                entries += k;
                return;
            }
            __syncwarp();
            if (lane < k) {
                const int bi = blist[bcnt - k + lane];
                const int pi = lane >> 1, h = lane & 1;
                reinterpret_cast<float*>(&bxy[pi])[h] = in.x[bi];
                reinterpret_cast<float*>(&bxy[pi])[2 + h] = in.y[bi];
                reinterpret_cast<float*>(&bm[pi])[h] = in.m[bi];
                reinterpret_cast<int*>(&bid[pi])[h] = bi;
            }
            __syncwarp();
            if (DIAG) {
                float f[BPL];
#pragma unroll
                for (int b = 0; b < BPL; ++b) f[b] = 0.0f;
                for (int e = 0; e < k; ++e) {
                    const int2 ids = bid[e >> 1];
                    const int who = (e & 1) ? ids.y : ids.x;
                    const float4 q = bxy[e >> 1];
                    const float2 w = bm[e >> 1];
                    const float x = (e & 1) ? q.y : q.x;
                    const float y = (e & 1) ? q.w : q.z;
                    const float m = (e & 1) ? w.y : w.x;
#pragma unroll
                    for (int b = 0; b < BPL; ++b) {
                        if (who == j[b]) continue;  // own body
                        const float dx = x - px[b], dy = y - py[b];
                        f[b] -= m * rsqrtf(fmaf(dx, dx, fmaf(dy, dy, eps2)));
                    }
                }
#pragma unroll
                for (int b = 0; b < BPL; ++b) phi[b] += (double)f[b];
            } else {
                float ox[BPL], oy[BPL];
                bodies_sum<BPL>(bxy, bm, k, px, py, npx, npy, eps2, ox, oy);
#pragma unroll
                for (int b = 0; b < BPL; ++b) add_batch(b, ox[b], oy[b]);
            }
            bcnt -= k;
            entries += k;
        };
        // cells every group of the super-group accepts: straight to the cell list
        for (int base = 0; base < nacc; base += 32) {
            const int k = min(32, nacc - base);
            __syncwarp();
            if (lane < k) clist[ccnt + lane] = fl[kFrontierCap - 1 - (base + lane)];
            ccnt += k;
            __syncwarp();
            while (ccnt >= 32) flush_cells(32);
        }
        while (top > 0) {
            if (rounds == kMaxWalkRounds) {  // far beyond any valid tree: report, do not loop
                if (lane == 0) atomicOr(status, ST_TREE);
                break;
            }
            int k = min(32, top);
            if (top + 3 * k > STACK) {  // pop k, push <= 4k: keep top+3k <= STACK
                k = max((STACK - top) / 3, 0);
                if (k == 0) {
                    overflow = true;
                    break;
                }
            }
            __syncwarp();
            const int node = lane < k ? stack[top - 1 - lane] : -1;
            top -= k;
            ++rounds;
            tested += k;
            int cat = -1;  // 0 approximate, 1 leaf bodies, 2 open
            int4 D = make_int4(0, 0, 0, 0);
            // Distance from the node's centre of mass to the group's bodies:
            // the group box gives a lower bound; the exact minimum over the
            // group's bodies is needed only when the box test is inconclusive,
            // i.e. d_box <= ropen < d_box + box diagonal, for some lane.
            float4 A = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            // the children's record is loaded after the decision, for the
            // opened nodes only (loading it with A and D, for every tested node
            // or only where the box test already opens the node, measured slower)
            int4 C = make_int4(kNoChild, kNoChild, kNoChild, kNoChild);
            float d2 = 0.0f;
            bool need = false;
            if (node >= 0) {
                A = recA[kRecStride * node];
                D = recD[kRecStride * node];
                if (ESTIMATE) A.w = __int_as_float(D.w);  // bootstrap opening radius
                const float ddx = fmaxf(fmaxf(gx0 - A.x, A.x - gx1), 0.0f);
                const float ddy = fmaxf(fmaxf(gy0 - A.y, A.y - gy1), 0.0f);
                d2 = fmaf(ddx, ddx, ddy * ddy);
                if (d2 <= A.w) {
                    const float reach = sqrt_approx(d2) + gdiag;
                    need = reach * reach > A.w * kRuleMargin;
                }
            }
            if (__any_sync(kFull, need)) {
                if (need) {
                    // an extreme body within the opening radius: the node is opened
                    const float4 ge = *gext;
                    float dx = gx0 - A.x, dy = ge.x - A.y;
                    float ub = fmaf(dx, dx, dy * dy);
                    dx = gx1 - A.x;
                    dy = ge.y - A.y;
                    ub = fminf(ub, fmaf(dx, dx, dy * dy));
                    dx = ge.z - A.x;
                    dy = gy0 - A.y;
                    ub = fminf(ub, fmaf(dx, dx, dy * dy));
                    dx = ge.w - A.x;
                    dy = gy1 - A.y;
                    ub = fminf(ub, fmaf(dx, dx, dy * dy));
                    if (ub <= A.w) {
                        d2 = ub;
                        need = false;
                    }
                }
                unsigned nm = __ballot_sync(kFull, need);
                if (__popc(nm) > kSerialExactLanes) {
                    // every lane: its node against the group's bodies, two at a
                    // time in FP32x2 (per component the scalar operations)
                    float2 e2 = make_float2(__int_as_float(0x7f800000), __int_as_float(0x7f800000));
                    const float2 nax = make_float2(-A.x, -A.x), nay = make_float2(-A.y, -A.y);
#pragma unroll 8
                    for (int e = 0; e < GW / 2; ++e) {
                        const float4 q = gp[e];
                        const float2 dx = __fadd2_rn(make_float2(q.x, q.y), nax);
                        const float2 dy = __fadd2_rn(make_float2(q.z, q.w), nay);
                        const float2 r = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
                        e2.x = fminf(e2.x, r.x);
                        e2.y = fminf(e2.y, r.y);
                    }
                    if (need) d2 = fminf(e2.x, e2.y);
                } else {
                    while (nm) {
                        const int src = __ffs(nm) - 1;
                        nm &= nm - 1;
                        const float cx = __shfl_sync(kFull, A.x, src);
                        const float cy = __shfl_sync(kFull, A.y, src);
                        float e2 = __int_as_float(0x7f800000);
#pragma unroll
                        for (int b = 0; b < BPL; ++b) {
                            const float dx = px[b] - cx, dy = py[b] - cy;
                            e2 = fminf(e2, fmaf(dx, dx, dy * dy));
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) e2 = fminf(e2, __shfl_xor_sync(kFull, e2, o));
                        if (lane == src) d2 = e2;
                    }
                }
            }
            if (node >= 0) {
                bool acc = d2 > A.w;
                if (acc && !ESTIMATE && !DIAG)
                    acc = __int_as_float(D.z) <= aa * kRuleMargin * d2 * d2 * sqrt_approx(d2);
                cat = acc ? 0 : (D.y <= BUCKET ? 1 : 2);
            }
            unsigned mc = __ballot_sync(kFull, cat == 0);
            if (cat == 0) clist[ccnt + __popc(mc & lt)] = node;
            ccnt += __popc(mc);
            if (cat == 2) C = recC[node];
            const int cs[4] = {C.x, C.y, C.z, C.w};
            int nb = cat == 1 ? D.y : 0, nn = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                nb += (cs[q] != kNoChild && cs[q] < 0);
                nn += (cs[q] >= 0);
            }
            int tot;
            const int off = warp_excl_scan(nb | (nn << 16), &tot);
            const int boff = off & 0xffff, noff = off >> 16;
            const int btot = tot & 0xffff, ntot = tot >> 16;
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
            peak = max(peak, top);
            __syncwarp();
            while (ccnt >= 32) flush_cells(32);
            while (bcnt >= 32) flush_bodies(32);
        }
        if (ccnt > 0) flush_cells(ccnt);
        if (bcnt > 0) flush_bodies(bcnt);
        if (sharing && ogr->w) {
            const bool redo = ows->w != 0;
            if (!redo) combine();
            if (redo) {  // out of room: the group again, unshared, before any other
                retry = ogr->z;
                __syncwarp();
                continue;
            }
        }
        if (lane == 0) {
            if (overflow) atomicOr(status, ST_STACK);
            atomicMax(max_stack, peak);
            if (!ESTIMATE && !DIAG) {
                atomicAdd(max_stack + 1, rounds);
                atomicAdd(max_stack + 2, tested);
            }
        }
        if (!ESTIMATE && !DIAG) {
            my_inter += (unsigned long long)(entries * cnt);
            my_cinter += (unsigned long long)(centries * cnt);
            if (hv.cost && lane == 0) atomicAdd(hv.cost + sg, (unsigned long long)(entries * cnt));
        }
        float wl = 0.0f, wr = 0.0f, wb = 0.0f, wt = 0.0f;  // new positions' box, from the origin
#pragma unroll
        for (int b = 0; b < BPL; ++b) {
            if (!valid[b]) continue;
            const int jb = j[b];
            const float gax = G * (MIXED ? ax[b] - cax[b] : ax[b]);
            const float gay = G * (MIXED ? ay[b] - cay[b] : ay[b]);
            if (DIAG) {
                pot[jb] = (double)G * phi[b];
                continue;
            }
            if (ESTIMATE) {
                in.amag[jb] = sqrtf(gax * gax + gay * gay);
                continue;
            }
            float vx = fmaf(dt, gax, in.vx[jb]);
            float vy = fmaf(dt, gay, in.vy[jb]);
            if (MIXED) {
                // x_hi + x_lo += d*dt*v with an error-free sum (TwoSum), renormalised
                float inc = ddt * vx, hx = px[b], s = hx + inc, bb = s - hx;
                float e = (hx - (s - bb)) + (inc - bb);
                float lo2 = in.xlo[jb] + e, h2 = s + lo2;
                const float nx = h2;
                out.x[jb] = h2;
                out.xlo[jb] = lo2 - (h2 - s);
                inc = ddt * vy;
                hx = py[b];
                s = hx + inc;
                bb = s - hx;
                e = (hx - (s - bb)) + (inc - bb);
                lo2 = in.ylo[jb] + e;
                h2 = s + lo2;
                out.y[jb] = h2;
                out.ylo[jb] = lo2 - (h2 - s);
                fold.check(nx, h2);
                wl = fminf(wl, nx);
                wr = fmaxf(wr, nx);
                wb = fminf(wb, h2);
                wt = fmaxf(wt, h2);
            } else {
                const float nx = fmaf(ddt, vx, px[b]), ny = fmaf(ddt, vy, py[b]);
                out.x[jb] = nx;
                out.y[jb] = ny;
                fold.check(nx, ny);
                wl = fminf(wl, nx);
                wr = fmaxf(wr, nx);
                wb = fminf(wb, ny);
                wt = fmaxf(wt, ny);
            }
            out.vx[jb] = vx;
            out.vy[jb] = vy;
            out.m[jb] = in.m[jb];
            out.id[jb] = in.id[jb];
            out.ax[jb] = gax;
            out.ay[jb] = gay;
            out.amag[jb] = sqrtf(gax * gax + gay * gay);
            out.gcost[jb] = (int)min(entries, 1ll << 30);  // next step's heavy-group estimate
        }
        if (folding) fold.group(sg, wl, wr, wb, wt);
    }
    if (folding) fold.finish();
    if (!ESTIMATE && !DIAG && lane == 0 && my_inter) {
        atomicAdd(inter_total, my_inter);
        atomicAdd(inter_total + 1, my_cinter);  // of which body-cell
    }
}

}  // namespace ssg
