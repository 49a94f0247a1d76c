/* Test infrastructure (oracle), never shipped.  CPU restatement of the
 * reference's 2D Barnes-Hut step (pentilm/StellarSolver kernels.cu), used only
 * as the checker in tests/, by __graft_entry__.smoke() and as the timed CPU
 * baseline in bench.py.  Nothing in the product path links this library.
 *
 * Float arithmetic is written op by op and built with -ffp-contract=off, so
 * every value below is a fixed function of its inputs.  Parity with the
 * reference is pinned by tests/golden/ fixtures produced by running the
 * reference's own kernels.cu (compiled for the host, oracle/ref_emu).
 *
 * Conventions shared with the engine:
 *   keys   : 64-bit quadrant keys, 2 bits per level, level 1 in bits 63..62.
 *            digit = (x < mid_x) | (y < mid_y) << 1, mid = (lo + hi) * 0.5f,
 *            i.e. the reference's child slot order (kernels.cu:144-157).
 *   tree   : binary radix tree over the sorted keys with Karras numbering
 *            (internal node i has one end of its body range at i; node 0 is
 *            the root).  Child encoding: >= 0 internal node, < 0 leaf ~pos.
 *            The quadtree is that tree with a node merged into its parent when
 *            both split the same 2-bit digit.
 */
#ifndef SSG_ORACLE_H
#define SSG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (match the engine's) */
#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_DUPLICATE_KEYS 2
#define ORC_ERR_NONFINITE 3

/* box = {left, right, bottom, top}: min/max of x and y merged into a box that
 * starts at (0,0,0,0) (kernels.cu:51-58, 62-114). */
int orc_bbox(int n, const float* x, const float* y, float* box);

/* 32-level float bisection keys (kernels.cu:137-185). */
void orc_keys(int n, const float* x, const float* y, const float* box, uint64_t* keys);

/* Stable ascending sort of keys; perm[j] = index of the j-th smallest key.
 * Returns the number of adjacent equal keys after sorting. */
int orc_sort_keys(int n, const uint64_t* keys, uint32_t* perm);

/* Binary radix tree over sorted, distinct keys (n >= 2).  Arrays of n-1:
 * left/right children, split bit (leading equal bits of the node's range),
 * first/last body position, parent (-1 at the root).  leaf_parent has n
 * entries.  qmerged[i] = 1 when node i is folded into its parent quadtree
 * node.  Returns ORC_OK or ORC_ERR_DUPLICATE_KEYS. */
int orc_build_tree(int n, const uint64_t* skeys, int32_t* left, int32_t* right,
                   int32_t* split_bit, int32_t* first, int32_t* last, int32_t* parent,
                   int32_t* leaf_parent, uint8_t* qmerged);

/* Mass sums of every binary node, children combined as left + right in float
 * (body term = (m, m*x, m*y)); com = sum / mass (IEEE division). */
void orc_node_sums(int n, const float* sx, const float* sy, const float* sm,
                   const int32_t* left, const int32_t* right, float* node_m, float* node_mx,
                   float* node_my, float* node_cx, float* node_cy);

/* Quadtree children of every non-merged binary node: qchild[4*i + k], k < 4,
 * in key order, INT32_MIN for an unused slot. */
void orc_quad_children(int n, const int32_t* left, const int32_t* right,
                       const int32_t* split_bit, const uint8_t* qmerged, int32_t* qchild);

/* Reference force walk (kernels.cu:340-435) on the quadtree: groups of 32
 * consecutive sorted bodies, a cell at level L >= 2 is approximated iff every
 * body of the group has dp_L <= dx*dx + dy*dy + eps2 with
 * dp_L = fl(fl(r*r)/theta) * 4^-(L-1), r = fl((right-left)*0.5); cells at
 * level <= 1 are always opened; body children always interact.  Output is in
 * sorted order.  Returns the number of interactions (body-node pairs). */
int64_t orc_walk_ref(int n, const float* sx, const float* sy, const float* sm,
                     const int32_t* split_bit, const int32_t* qchild, const float* node_m,
                     const float* node_cx, const float* node_cy, const float* box, float theta,
                     float eps2, float* sax, float* say);

/* One whole reference step in the caller's body order: bbox, keys, sort,
 * tree, centre of mass, force walk, then v += dt*a; x += (d*dt)*v
 * (kernels.cu:522-537).  ax/ay receive the accelerations.  *interactions
 * (optional) receives the walk's interaction count. */
int orc_step_ref(int n, float* x, float* y, float* vx, float* vy, const float* m, float* ax,
                 float* ay, float theta, float eps2, float dt, float damp,
                 int64_t* interactions);

/* FP64 direct sum: for each of ns targets idx[k], a = G * sum_j m_j d / (|d|^2+eps2)^1.5 */
void orc_direct_f64(int n, const float* x, const float* y, const float* m, int ns,
                    const int32_t* idx, double eps2, double G, double* ax, double* ay);

/* Same, with positions given as hi + lo float pairs (either lo may be NULL). */
void orc_direct_f64_hilo(int n, const float* xh, const float* xl, const float* yh,
                         const float* yl, const float* m, int ns, const int32_t* idx,
                         double eps2, double G, double* ax, double* ay);

/* FP64 energy and momentum: out = {kinetic, potential, px, py}; O(n^2). */
void orc_energy_f64(int n, const float* x, const float* y, const float* vx, const float* vy,
                    const float* m, double eps2, double G, double* out);

/* CPU restatement of the engine's PLAIN-mode group walk: quadrupoles, leaf
 * buckets, geometric + relative opening rule (see oracle.c; aold = |a| of the
 * previous step in sorted order, NULL for the geometric-only bootstrap pass;
 * quadrupole = 0 evaluates accepted cells as monopoles, as the engine's
 * bootstrap pass does; group = bodies per walk group, 32 or 64).  Output in sorted order; returns the interaction count. */
int64_t orc_walk_acc(int n, const float* sx, const float* sy, const float* sm,
                     const uint64_t* skeys, const int32_t* left, const int32_t* right,
                     const int32_t* split, const int32_t* first, const int32_t* last,
                     const int32_t* qchild, const float* box, float theta, float eps2, float G,
                     int bucket, float alpha, const float* aold, int quadrupole, int group,
                     float* sax, float* say);

/* The engine's shared walk frontiers (k_frontier in bh_walk.cuh) checked on
 * the CPU, for one system: per super-group of `super` consecutive bodies the
 * nodes every group of it opens (not a leaf bucket, only node children, the
 * super-group box's farthest corner within the opening radius) are opened
 * once; frontier nodes every group accepts (the box's nearest point beyond the
 * radius, the relative rule at the smallest group scale taken 0.1 % low) go
 * to the groups untested.  Each group's accepted cells and direct bodies are
 * then compared between the root start and the frontier start, with the
 * decisions of orc_walk_acc.  stats[0] = groups whose sets differ (0 is the
 * claim), [1] = frontier nodes, [2] = accepted frontier cells, [3] = node
 * tests from the root, [4] = node tests from the frontiers. */
void orc_frontier_check(int n, const float* sx, const float* sy, const float* sm,
                        const uint64_t* skeys, const int32_t* left, const int32_t* right,
                        const int32_t* split, const int32_t* first, const int32_t* last,
                        const int32_t* qchild, const float* box, float theta, float G, int bucket,
                        float alpha, const float* aold, int group, int super, int64_t* stats);

/* Tree invariants (the engine's bh_check, restated for one system; the
 * reference's debug.cpp:23-174 on a binary radix tree): returns the mask of
 * failing checks, bits as BH_CHECK_* in include/stellar_bh.h.  Node arrays have
 * n - 1 entries; sm = masses in sorted order; id = caller index per position;
 * box = left, right, bottom, top. */
unsigned orc_check_tree(int n, const uint64_t* skeys, const int32_t* left, const int32_t* right,
                        const int32_t* parent, const int32_t* leaf_parent, const int32_t* first,
                        const int32_t* last, const float* sm, const float* node_m,
                        const int32_t* id, const float* box);

/* Headless point rendering (the engine's bh_render restated): counts of
 * points per pixel, column floor((x - x0) * sx), row from the bottom, with
 * sx = width / (x1 - x0); then RGBA8 with colour min(1, 0.1 c) and alpha
 * min(1, 0.5 + 0.01 c) rounded to 1/255.  rgba: width*height*4, top row first. */
void orc_render(int n, const float* x, const float* y, int width, int height, float x0, float x1,
                float y0, float y1, unsigned char* rgba);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
