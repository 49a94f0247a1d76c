// bh_check.cuh -- tree invariants of the last step, checked on the device.
//
// The reference checks its tree on the host after copying every array back
// (debug.cpp:23-174, called from BarnesHutParticleSystem.cpp:331-344):
// child counts add up, every body is a child exactly once, child indices are in
// range, `sorted` is a permutation, the box is ordered.  These kernels state
// the same invariants for the engine's binary radix tree and return one status
// word.  Every index is range-checked before it is dereferenced, so a broken
// tree is reported, never followed.
#pragma once

#include "bh_device.cuh"

namespace ssg {

// bits of the status word (mirrored by BH_CHECK_* in stellar_bh.h)
enum : unsigned {
    CK_COUNT = 1u,         // a node's range is not the union of its children's ranges
    CK_CHILD_SUM = 2u,     // positions as leaf children: not each position exactly once
    CK_CHILD_RANGE = 4u,   // a child index outside its system
    CK_PARENT = 8u,        // parent / leaf_parent does not point back
    CK_KEYS_SORTED = 16u,  // keys not ascending within a system
    CK_PERMUTATION = 32u,  // caller indices of the positions are not a permutation
    CK_BOX = 64u,          // left > right or bottom > top
    CK_MASS = 128u,        // a node's mass is not the sum of its children's
};

// One thread per position i: node i (i < the system's last position), or the
// single body of a one-body system.  acc[0] += positions seen as leaf children,
// acc[1] += number of leaf children.
static __global__ void k_check_nodes(int n, Segs segs, TreePtrs t, const float* __restrict__ sm,
                                     NodeSums ns, unsigned long long* __restrict__ acc,
                                     unsigned* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned f = 0;
    unsigned long long psum = 0, leaves = 0;
    if (i < n) {
        const int s = seg_of(segs, i);
        const int lo = segs.off[s], hi = segs.off[s + 1] - 1;
        if (i == hi) {
            if (lo == hi) {  // a one-body system: its body is no node's child
                psum = (unsigned long long)i;
                leaves = 1;
            }
        } else {
            const int a = t.first[i], b = t.last[i];
            if (a < lo || b > hi || a >= b || (a != i && b != i)) f |= CK_COUNT;
            const int ch[2] = {t.left[i], t.right[i]};
            int cf[2] = {0, 0}, cl[2] = {0, 0};
            float cm[2] = {0.0f, 0.0f};
            bool ok = true;
            for (int q = 0; q < 2; ++q) {
                const int c = ch[q];
                if (c == kNoChild) {
                    ok = false;
                } else if (c < 0) {
                    const int body = ~c;
                    if (body < lo || body > hi) {
                        ok = false;
                    } else {
                        psum += (unsigned long long)body;
                        leaves += 1;
                        if (t.leaf_parent[body] != i) f |= CK_PARENT;
                        cf[q] = cl[q] = body;
                        cm[q] = sm[body];
                    }
                } else if (c < lo || c >= hi) {
                    ok = false;
                } else {
                    if (t.parent[c] != i) f |= CK_PARENT;
                    cf[q] = t.first[c];
                    cl[q] = t.last[c];
                    cm[q] = ns.s0[c].x;
                }
            }
            if (!ok) {
                f |= CK_CHILD_RANGE;
            } else {
                if (cf[0] != a || cl[1] != b || cl[0] + 1 != cf[1]) f |= CK_COUNT;
                if (__fadd_rn(cm[0], cm[1]) != ns.s0[i].x) f |= CK_MASS;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        psum += __shfl_xor_sync(kFull, psum, o);
        leaves += __shfl_xor_sync(kFull, leaves, o);
        f |= __shfl_xor_sync(kFull, f, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (psum) atomicAdd(acc, psum);
        if (leaves) atomicAdd(acc + 1, leaves);
        if (f) atomicOr(flags, f);
    }
}

// One thread per position j: key order, caller index (counted in seen[]), box.
static __global__ void k_check_bodies(int n, Segs segs, const uint64_t* __restrict__ keys,
                                      const int* __restrict__ id, int* __restrict__ seen,
                                      const int* __restrict__ box_ord, unsigned* __restrict__ flags) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned f = 0;
    if (j < n) {
        const int s = seg_of(segs, j);
        const int lo = segs.off[s], hi = segs.off[s + 1] - 1;
        if (j < hi && keys[j] > keys[j + 1]) f |= CK_KEYS_SORTED;
        const int c = id[j];
        if (c < 0 || c >= n)
            f |= CK_PERMUTATION;
        else
            atomicAdd(seen + c, 1);
        if (j == lo) {
            const Box bx = load_box(box_ord, s);
            if (!(bx.l <= bx.r) || !(bx.b <= bx.t)) f |= CK_BOX;
        }
    }
    f = __reduce_or_sync(kFull, f);
    if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

static __global__ void k_check_seen(int n, const int* __restrict__ seen, unsigned* __restrict__ flags) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const bool bad = j < n && seen[j] != 1;
    if (__any_sync(kFull, bad) && (threadIdx.x & 31) == 0) atomicOr(flags, CK_PERMUTATION);
}

}  // namespace ssg
