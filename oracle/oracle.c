/* Test infrastructure (oracle), never shipped.  CPU restatement of the
 * reference's 2D Barnes-Hut step; see oracle.h for the conventions.  Each
 * function cites the part of the reference (pentilm/StellarSolver) it restates.
 * Parity against the reference itself is pinned by the golden fixtures in
 * tests/golden/, produced by running the reference's kernels.cu on the host.
 */
#include "oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

int orc_num_threads(void) { return omp_get_max_threads(); }

/* kernels.cu:51-58 (box reset to 0) and :62-114 (min/max merge). */
int orc_bbox(int n, const float* x, const float* y, float* box) {
    float l = 0.0f, r = 0.0f, b = 0.0f, t = 0.0f;
    for (int i = 0; i < n; ++i) {
        if (!isfinite(x[i]) || !isfinite(y[i])) return ORC_ERR_NONFINITE;
        l = fminf(l, x[i]);
        r = fmaxf(r, x[i]);
        b = fminf(b, y[i]);
        t = fmaxf(t, y[i]);
    }
    box[0] = l;
    box[1] = r;
    box[2] = b;
    box[3] = t;
    return ORC_OK;
}

/* kernels.cu:137-185: per level, mid = 0.5*(lo+hi) (the double literal makes
 * no difference: halving a float sum is exact), digit bit 0 = (x < mid_x),
 * bit 1 = (y < mid_y); the body's half becomes the new interval. */
static uint64_t key_of(float px, float py, const float* box) {
    float l = box[0], r = box[1], b = box[2], t = box[3];
    uint64_t key = 0;
    for (int level = 0; level < 32; ++level) {
        float mx = (l + r) * 0.5f;
        float my = (b + t) * 0.5f;
        unsigned c = 0;
        if (px < mx) {
            c |= 1u;
            r = mx;
        } else {
            l = mx;
        }
        if (py < my) {
            c |= 2u;
            t = my;
        } else {
            b = my;
        }
        key = (key << 2) | c;
    }
    return key;
}

void orc_keys(int n, const float* x, const float* y, const float* box, uint64_t* keys) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) keys[i] = key_of(x[i], y[i], box);
}

/* Leaves in DFS order over child slots 0..3 (sort_kernel, kernels.cu:292-336)
 * are the bodies in ascending key order.  LSD radix sort, 8 passes of 8 bits. */
int orc_sort_keys(int n, const uint64_t* keys, uint32_t* perm) {
    if (n <= 0) return 0;
    uint64_t* k0 = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n);
    uint64_t* k1 = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n);
    uint32_t* p1 = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    memcpy(k0, keys, sizeof(uint64_t) * (size_t)n);
    for (int i = 0; i < n; ++i) perm[i] = (uint32_t)i;
    uint32_t* p0 = perm;
    for (int pass = 0; pass < 8; ++pass) {
        int shift = 8 * pass;
        size_t cnt[257];
        memset(cnt, 0, sizeof cnt);
        for (int i = 0; i < n; ++i) cnt[((k0[i] >> shift) & 255u) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (int i = 0; i < n; ++i) {
            size_t dst = cnt[(k0[i] >> shift) & 255u]++;
            k1[dst] = k0[i];
            p1[dst] = p0[i];
        }
        uint64_t* tk = k0;
        k0 = k1;
        k1 = tk;
        uint32_t* tp = p0;
        p0 = p1;
        p1 = tp;
    }
    /* 8 passes: an even count, so the result is back in `perm` */
    int dups = 0;
    for (int i = 1; i < n; ++i) dups += (k0[i] == k0[i - 1]);
    free(k0);
    free(k1);
    free(p1);
    return dups;
}

static int lcp_bits(uint64_t a, uint64_t b) { return a == b ? 64 : __builtin_clzll(a ^ b); }

typedef struct {
    const uint64_t* k;
    int32_t *left, *right, *split, *first, *last, *parent, *leaf_parent;
} TreeCtx;

/* Internal node `id` covers sorted bodies [a, b], a < b. */
static void build_node(TreeCtx* t, int a, int b, int id, int parent) {
    int p = lcp_bits(t->k[a], t->k[b]);
    int bit = 63 - p;
    int lo = a, hi = b; /* bit of k[lo] is 0, bit of k[hi] is 1 */
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if ((t->k[mid] >> bit) & 1u)
            hi = mid;
        else
            lo = mid;
    }
    int g = lo;
    t->split[id] = p;
    t->first[id] = a;
    t->last[id] = b;
    t->parent[id] = parent;
    if (g == a) {
        t->left[id] = ~a;
        t->leaf_parent[a] = id;
    } else {
        t->left[id] = g;
        build_node(t, a, g, g, id);
    }
    if (g + 1 == b) {
        t->right[id] = ~b;
        t->leaf_parent[b] = id;
    } else {
        t->right[id] = g + 1;
        build_node(t, g + 1, b, g + 1, id);
    }
}

/* The reference's tree (kernels.cu:117-271) holds one cell per key prefix
 * shared by >= 2 bodies; the binary radix tree below has the same leaves and,
 * after the digit merge, exactly the reference's branching cells (chain cells
 * with one child are implicit: they carry their only child's sums). */
int orc_build_tree(int n, const uint64_t* skeys, int32_t* left, int32_t* right,
                   int32_t* split_bit, int32_t* first, int32_t* last, int32_t* parent,
                   int32_t* leaf_parent, uint8_t* qmerged) {
    if (n < 2) return ORC_ERR_ARG;
    for (int i = 1; i < n; ++i)
        if (skeys[i] == skeys[i - 1]) return ORC_ERR_DUPLICATE_KEYS;
    TreeCtx t = {skeys, left, right, split_bit, first, last, parent, leaf_parent};
    build_node(&t, 0, n - 1, 0, -1);
    for (int i = 0; i < n - 1; ++i) {
        int s = split_bit[i];
        qmerged[i] = (uint8_t)(i != 0 && (s & 1) && split_bit[parent[i]] == s - 1);
    }
    return ORC_OK;
}

typedef struct {
    const float *sx, *sy, *sm;
    const int32_t *left, *right;
    float *m, *mx, *my;
} SumCtx;

static void child_sums(const SumCtx* c, int32_t ch, float* m, float* mx, float* my);

static void node_sums(const SumCtx* c, int id) {
    float lm, lmx, lmy, rm, rmx, rmy;
    child_sums(c, c->left[id], &lm, &lmx, &lmy);
    child_sums(c, c->right[id], &rm, &rmx, &rmy);
    c->m[id] = lm + rm;
    c->mx[id] = lmx + rmx;
    c->my[id] = lmy + rmy;
}

static void child_sums(const SumCtx* c, int32_t ch, float* m, float* mx, float* my) {
    if (ch < 0) {
        int j = ~ch;
        float mj = c->sm[j];
        *m = mj;
        *mx = mj * c->sx[j]; /* kernels.cu:180-181: mass*x */
        *my = mj * c->sy[j];
    } else {
        node_sums(c, ch);
        *m = c->m[ch];
        *mx = c->mx[ch];
        *my = c->my[ch];
    }
}

/* kernels.cu:180-183 (sums) and :275-288 (x /= mass). */
void orc_node_sums(int n, const float* sx, const float* sy, const float* sm,
                   const int32_t* left, const int32_t* right, float* node_m, float* node_mx,
                   float* node_my, float* node_cx, float* node_cy) {
    if (n < 2) return;
    SumCtx c = {sx, sy, sm, left, right, node_m, node_mx, node_my};
    node_sums(&c, 0);
    for (int i = 0; i < n - 1; ++i) {
        node_cx[i] = node_mx[i] / node_m[i];
        node_cy[i] = node_my[i] / node_m[i];
    }
}

void orc_quad_children(int n, const int32_t* left, const int32_t* right,
                       const int32_t* split_bit, const uint8_t* qmerged, int32_t* qchild) {
    (void)split_bit;
    for (int i = 0; i < n - 1; ++i) {
        int k = 0;
        int32_t* out = qchild + 4 * (size_t)i;
        for (int s = 0; s < 4; ++s) out[s] = INT32_MIN;
        if (qmerged[i]) continue;
        int32_t cs[2] = {left[i], right[i]};
        for (int s = 0; s < 2; ++s) {
            int32_t c = cs[s];
            if (c >= 0 && qmerged[c]) {
                out[k++] = left[c];
                out[k++] = right[c];
            } else {
                out[k++] = c;
            }
        }
    }
}

/* kernels.cu:340-435: one group = 32 consecutive sorted bodies (a warp).
 * dp for a cell at level L is radius^2/theta scaled by 0.25 per level below
 * the root's children (:349, :376, :395); the test is dp <= dx*dx+dy*dy+eps2
 * on every lane (:405-406); the force is m * d * rsqrt(r)^3 (:407-411). */
int64_t orc_walk_ref(int n, const float* sx, const float* sy, const float* sm,
                     const int32_t* split_bit, const int32_t* qchild, const float* node_m,
                     const float* node_cx, const float* node_cy, const float* box, float theta,
                     float eps2, float* sax, float* say) {
    if (n == 1) {
        sax[0] = 0.0f;
        say[0] = 0.0f;
        return 0;
    }
    if (n < 1) return 0;
    float radius = (box[1] - box[0]) * 0.5f;
    float dp1 = (radius * radius) / theta;
    int groups = (n + 31) / 32;
    int64_t total = 0;
#pragma omp parallel reduction(+ : total)
    {
        int cap = 1024;
        int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
#pragma omp for schedule(dynamic, 16)
        for (int g = 0; g < groups; ++g) {
            int g0 = 32 * g;
            int cnt = n - g0 < 32 ? n - g0 : 32;
            float px[32], py[32], ax[32], ay[32], rr[32];
            for (int k = 0; k < cnt; ++k) {
                px[k] = sx[g0 + k];
                py[k] = sy[g0 + k];
                ax[k] = 0.0f;
                ay[k] = 0.0f;
            }
            int64_t inter = 0;
            int top = 0;
            /* the root is never approximated unless its chain reaches level 2 */
            int32_t pending[1] = {0};
            for (int pi = 0; pi < 1; ++pi) {
                int32_t q = pending[pi];
                int L = split_bit[q] >> 1;
                int accept = 0;
                if (L >= 2) {
                    float dp = ldexpf(dp1, -2 * (L - 1));
                    accept = 1;
                    for (int k = 0; k < cnt; ++k) {
                        float dx = node_cx[q] - px[k];
                        float dy = node_cy[q] - py[k];
                        float r = dx * dx;
                        r = r + dy * dy;
                        r = r + eps2;
                        rr[k] = r;
                        accept &= (dp <= r);
                    }
                }
                if (accept) {
                    for (int k = 0; k < cnt; ++k) {
                        float dx = node_cx[q] - px[k];
                        float dy = node_cy[q] - py[k];
                        float ri = 1.0f / sqrtf(rr[k]);
                        float f = node_m[q] * ri;
                        f = f * ri;
                        f = f * ri;
                        ax[k] = ax[k] + f * dx;
                        ay[k] = ay[k] + f * dy;
                    }
                    inter += cnt;
                } else {
                    stack[top++] = q;
                }
            }
            while (top > 0) {
                int32_t node = stack[--top];
                for (int s = 0; s < 4; ++s) {
                    int32_t c = qchild[4 * (size_t)node + s];
                    if (c == INT32_MIN) continue;
                    float cxv, cyv, mv;
                    int L = 0;
                    if (c < 0) {
                        cxv = sx[~c];
                        cyv = sy[~c];
                        mv = sm[~c];
                    } else {
                        cxv = node_cx[c];
                        cyv = node_cy[c];
                        mv = node_m[c];
                        L = split_bit[c] >> 1;
                    }
                    int accept = 1;
                    float dp = L >= 2 ? ldexpf(dp1, -2 * (L - 1)) : 0.0f;
                    for (int k = 0; k < cnt; ++k) {
                        float dx = cxv - px[k];
                        float dy = cyv - py[k];
                        float r = dx * dx;
                        r = r + dy * dy;
                        r = r + eps2;
                        rr[k] = r;
                        if (c >= 0) accept &= (L >= 2) && (dp <= r);
                    }
                    if (accept) {
                        for (int k = 0; k < cnt; ++k) {
                            float dx = cxv - px[k];
                            float dy = cyv - py[k];
                            float ri = 1.0f / sqrtf(rr[k]);
                            float f = mv * ri;
                            f = f * ri;
                            f = f * ri;
                            ax[k] = ax[k] + f * dx;
                            ay[k] = ay[k] + f * dy;
                        }
                        inter += cnt;
                    } else {
                        if (top == cap) {
                            cap *= 2;
                            stack = (int32_t*)realloc(stack, sizeof(int32_t) * (size_t)cap);
                        }
                        stack[top++] = c;
                    }
                }
            }
            for (int k = 0; k < cnt; ++k) {
                sax[g0 + k] = ax[k];
                say[g0 + k] = ay[k];
            }
            total += inter;
        }
        free(stack);
    }
    return total;
}

int orc_step_ref(int n, float* x, float* y, float* vx, float* vy, const float* m, float* ax,
                 float* ay, float theta, float eps2, float dt, float damp,
                 int64_t* interactions) {
    if (n < 1) return ORC_ERR_ARG;
    float box[4];
    int st = orc_bbox(n, x, y, box);
    if (st) return st;
    size_t N = (size_t)n;
    uint64_t* keys = (uint64_t*)malloc(8 * N);
    uint64_t* skeys = (uint64_t*)malloc(8 * N);
    uint32_t* perm = (uint32_t*)malloc(4 * N);
    float* sx = (float*)malloc(4 * N);
    float* sy = (float*)malloc(4 * N);
    float* sm = (float*)malloc(4 * N);
    float* sax = (float*)malloc(4 * N);
    float* say = (float*)malloc(4 * N);
    size_t nn = N > 1 ? N - 1 : 1;
    int32_t* left = (int32_t*)malloc(4 * nn);
    int32_t* right = (int32_t*)malloc(4 * nn);
    int32_t* split = (int32_t*)malloc(4 * nn);
    int32_t* first = (int32_t*)malloc(4 * nn);
    int32_t* last = (int32_t*)malloc(4 * nn);
    int32_t* parent = (int32_t*)malloc(4 * nn);
    int32_t* lparent = (int32_t*)malloc(4 * N);
    uint8_t* qm = (uint8_t*)malloc(nn);
    int32_t* qc = (int32_t*)malloc(16 * nn);
    float* nm = (float*)malloc(4 * nn);
    float* nmx = (float*)malloc(4 * nn);
    float* nmy = (float*)malloc(4 * nn);
    float* ncx = (float*)malloc(4 * nn);
    float* ncy = (float*)malloc(4 * nn);
    int64_t inter = 0;

    orc_keys(n, x, y, box, keys);
    orc_sort_keys(n, keys, perm);
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) {
        uint32_t i = perm[j];
        skeys[j] = keys[i];
        sx[j] = x[i];
        sy[j] = y[i];
        sm[j] = m[i];
    }
    if (n >= 2) {
        st = orc_build_tree(n, skeys, left, right, split, first, last, parent, lparent, qm);
        if (st == ORC_OK) {
            orc_node_sums(n, sx, sy, sm, left, right, nm, nmx, nmy, ncx, ncy);
            orc_quad_children(n, left, right, split, qm, qc);
            inter = orc_walk_ref(n, sx, sy, sm, split, qc, nm, ncx, ncy, box, theta, eps2, sax,
                                 say);
        }
    } else {
        sax[0] = 0.0f;
        say[0] = 0.0f;
    }
    if (st == ORC_OK) {
#pragma omp parallel for schedule(static)
        for (int j = 0; j < n; ++j) {
            ax[perm[j]] = sax[j];
            ay[perm[j]] = say[j];
        }
        /* kernels.cu:529-533 */
        float ddt = damp * dt;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            vx[i] = vx[i] + dt * ax[i];
            vy[i] = vy[i] + dt * ay[i];
            x[i] = x[i] + ddt * vx[i];
            y[i] = y[i] + ddt * vy[i];
        }
    }
    if (interactions) *interactions = inter;
    free(keys);
    free(skeys);
    free(perm);
    free(sx);
    free(sy);
    free(sm);
    free(sax);
    free(say);
    free(left);
    free(right);
    free(split);
    free(first);
    free(last);
    free(parent);
    free(lparent);
    free(qm);
    free(qc);
    free(nm);
    free(nmx);
    free(nmy);
    free(ncx);
    free(ncy);
    return st;
}

void orc_direct_f64_hilo(int n, const float* xh, const float* xl, const float* yh,
                         const float* yl, const float* m, int ns, const int32_t* idx,
                         double eps2, double G, double* ax, double* ay) {
#pragma omp parallel for schedule(dynamic, 8)
    for (int k = 0; k < ns; ++k) {
        int i = idx[k];
        double xi = (double)xh[i] + (xl ? (double)xl[i] : 0.0);
        double yi = (double)yh[i] + (yl ? (double)yl[i] : 0.0);
        double sx = 0.0, sy = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            double dx = (double)xh[j] + (xl ? (double)xl[j] : 0.0) - xi;
            double dy = (double)yh[j] + (yl ? (double)yl[j] : 0.0) - yi;
            double r2 = dx * dx + dy * dy + eps2;
            double inv = 1.0 / (r2 * sqrt(r2));
            sx += (double)m[j] * dx * inv;
            sy += (double)m[j] * dy * inv;
        }
        ax[k] = G * sx;
        ay[k] = G * sy;
    }
}

void orc_direct_f64(int n, const float* x, const float* y, const float* m, int ns,
                    const int32_t* idx, double eps2, double G, double* ax, double* ay) {
    orc_direct_f64_hilo(n, x, NULL, y, NULL, m, ns, idx, eps2, G, ax, ay);
}

void orc_energy_f64(int n, const float* x, const float* y, const float* vx, const float* vy,
                    const float* m, double eps2, double G, double* out) {
    double ke = 0.0, pe = 0.0, px = 0.0, py = 0.0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : ke, pe, px, py)
    for (int i = 0; i < n; ++i) {
        double mi = m[i];
        ke += 0.5 * mi * ((double)vx[i] * vx[i] + (double)vy[i] * vy[i]);
        px += mi * vx[i];
        py += mi * vy[i];
        double s = 0.0;
        for (int j = i + 1; j < n; ++j) {
            double dx = (double)x[j] - x[i];
            double dy = (double)y[j] - y[i];
            s += (double)m[j] / sqrt(dx * dx + dy * dy + eps2);
        }
        pe -= G * mi * s;
    }
    out[0] = ke;
    out[1] = pe;
    out[2] = px;
    out[3] = py;
}

/* ------------------------------------------------------------------------
 * CPU restatement of the engine's PLAIN-mode walk (no reference counterpart:
 * the reference has one monopole walk).  Checks the GPU walk and its opening
 * rule against the FP64 direct sum.  Per group of 32 consecutive sorted
 * bodies, a node is approximated by its quadrupole expansion iff
 *   geometric: d > l/theta + |COM - cell centre|, where d is the distance
 *              from the COM to the group's box when that already decides
 *              (box distance > r, or box distance + box diagonal <= r), else
 *              min_j |COM - p_j| (l = larger side of the node's cell), and
 *   relative : G M l^3 <= alpha * a_g * d^5 with the same d,
 *              a_g = max(min_j |a_old_j|, 0.1 * mean_j |a_old_j|)
 *              (skipped when aold == NULL or alpha <= 0);
 * otherwise a node of <= bucket bodies interacts body by body and a larger
 * node is opened.  Float arithmetic, as on the GPU.
 * ---------------------------------------------------------------------- */
typedef struct {
    float m, cx, cy, sxx, sxy, syy;
} Mom;

static void acc_moments(int id, const int32_t* left, const int32_t* right, const float* sx,
                        const float* sy, const float* sm, Mom* out) {
    Mom c[2];
    int32_t ch[2] = {left[id], right[id]};
    for (int s = 0; s < 2; ++s) {
        if (ch[s] < 0) {
            int b = ~ch[s];
            c[s].m = sm[b];
            c[s].cx = sx[b];
            c[s].cy = sy[b];
            c[s].sxx = c[s].sxy = c[s].syy = 0.0f;
        } else {
            acc_moments(ch[s], left, right, sx, sy, sm, out);
            c[s] = out[ch[s]];
        }
    }
    Mom r;
    r.m = c[0].m + c[1].m;
    float w = r.m > 0.0f ? c[1].m / r.m : 0.5f;
    r.cx = w * (c[1].cx - c[0].cx) + c[0].cx;
    r.cy = w * (c[1].cy - c[0].cy) + c[0].cy;
    float ax = c[0].cx - r.cx, ay = c[0].cy - r.cy, bx = c[1].cx - r.cx, by = c[1].cy - r.cy;
    r.sxx = c[0].sxx + c[1].sxx + c[0].m * ax * ax + c[1].m * bx * bx;
    r.sxy = c[0].sxy + c[1].sxy + c[0].m * ax * ay + c[1].m * bx * by;
    r.syy = c[0].syy + c[1].syy + c[0].m * ay * ay + c[1].m * by * by;
    out[id] = r;
}

static void p2p_cpu(float bx, float by, float bm, float px, float py, float eps2, float* ax,
                    float* ay) {
    float dx = bx - px, dy = by - py;
    float u = dx * dx + dy * dy + eps2;
    float ri = u > 0.0f ? 1.0f / sqrtf(u) : 0.0f;
    float f = bm * ri * ri * ri;
    *ax += f * dx;
    *ay += f * dy;
}

/* Opening radius^2 and relative-rule numerator G M l^3 of every node: l the
 * node's cell side (the larger box side halved per level), ropen = l / theta +
 * |COM - cell centre| (the engine's k_records). */
static void open_radii(int n, const Mom* mom, const uint64_t* skeys, const int32_t* split,
                       const int32_t* first, const float* box, float theta, float G,
                       float* ropen2, float* qerr) {
    for (int i = 0; i < n - 1; ++i) {
        int L = split[i] >> 1;
        if (L > 32) L = 32;
        uint64_t pre = L > 0 ? skeys[first[i]] >> (64 - 2 * L) : 0;
        unsigned long long ix = 0, iy = 0;
        for (int q = L - 1; q >= 0; --q) {
            unsigned d = (unsigned)(pre >> (2 * q)) & 3u;
            ix = (ix << 1) | ((d & 1u) ? 0ull : 1ull);
            iy = (iy << 1) | ((d & 2u) ? 0ull : 1ull);
        }
        double wx = (double)box[1] - box[0], wy = (double)box[3] - box[2];
        double sc = ldexp(1.0, -L);
        double x0 = box[0] + wx * sc * (double)ix, y0 = box[2] + wy * sc * (double)iy;
        double l = fmax(wx, wy) * sc;
        double dx = mom[i].cx - (x0 + 0.5 * wx * sc), dy = mom[i].cy - (y0 + 0.5 * wy * sc);
        double r = l / theta + sqrt(dx * dx + dy * dy);
        ropen2[i] = (float)(r * r);
        qerr[i] = (float)((double)G * mom[i].m * l * l * l);
    }
}

int64_t orc_walk_acc(int n, const float* sx, const float* sy, const float* sm,
                     const uint64_t* skeys, const int32_t* left, const int32_t* right,
                     const int32_t* split, const int32_t* first, const int32_t* last,
                     const int32_t* qchild, const float* box, float theta, float eps2, float G,
                     int bucket, float alpha, const float* aold, int quadrupole, int group,
                     float* sax, float* say) {
    if (n < 2) {
        for (int i = 0; i < n; ++i) sax[i] = say[i] = 0.0f;
        return 0;
    }
    Mom* mom = (Mom*)malloc(sizeof(Mom) * (size_t)(n - 1));
    acc_moments(0, left, right, sx, sy, sm, mom);
    float* ropen2 = (float*)malloc(sizeof(float) * (size_t)(n - 1));
    float* qerr = (float*)malloc(sizeof(float) * (size_t)(n - 1));
    open_radii(n, mom, skeys, split, first, box, theta, G, ropen2, qerr);
    const int relative = aold != NULL && alpha > 0.0f;
    if (group != 64) group = 32;  /* bodies per group: 32, or 64 (two per lane) */
    int groups = (n + group - 1) / group;
    int64_t total = 0;
#pragma omp parallel reduction(+ : total)
    {
        int cap = 4096;
        int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
#pragma omp for schedule(dynamic, 4)
        for (int g = 0; g < groups; ++g) {
            int g0 = group * g, cnt = n - g0 < group ? n - g0 : group;
            float px[64], py[64], ax[64], ay[64];
            float aa = INFINITY;
            if (relative) {
                float amin = INFINITY, amean = 0.0f;
                for (int k = 0; k < cnt; ++k) {
                    amin = fminf(amin, aold[g0 + k]);
                    amean += aold[g0 + k];
                }
                amean /= (float)cnt;
                aa = alpha * fmaxf(amin, 0.1f * amean);
            }
            float gx0 = sx[g0], gx1 = sx[g0], gy0 = sy[g0], gy1 = sy[g0];
            for (int k = 0; k < cnt; ++k) {
                px[k] = sx[g0 + k];
                py[k] = sy[g0 + k];
                ax[k] = ay[k] = 0.0f;
                gx0 = fminf(gx0, px[k]);
                gx1 = fmaxf(gx1, px[k]);
                gy0 = fminf(gy0, py[k]);
                gy1 = fmaxf(gy1, py[k]);
            }
            const float gdiag = sqrtf((gx1 - gx0) * (gx1 - gx0) + (gy1 - gy0) * (gy1 - gy0));
            int64_t entries = 0;
            int top = 0;
            stack[top++] = 0;
            while (top > 0) {
                int32_t node = stack[--top];
                float cx = mom[node].cx, cy = mom[node].cy;
                /* group-box lower bound; exact minimum only when inconclusive */
                float ddx = fmaxf(fmaxf(gx0 - cx, cx - gx1), 0.0f);
                float ddy = fmaxf(fmaxf(gy0 - cy, cy - gy1), 0.0f);
                float d2 = ddx * ddx + ddy * ddy;
                if (d2 <= ropen2[node]) {
                    float reach = sqrtf(d2) + gdiag;
                    if (reach * reach > ropen2[node]) {
                        d2 = INFINITY;
                        for (int k = 0; k < cnt; ++k) {
                            float dx = px[k] - cx, dy = py[k] - cy;
                            float q = dx * dx + dy * dy;
                            d2 = q < d2 ? q : d2;
                        }
                    }
                }
                int accept = d2 > ropen2[node];
                if (accept && relative) accept = qerr[node] <= aa * d2 * d2 * sqrtf(d2);
                if (accept) {
                    const Mom* M = &mom[node];
                    float T0 = 3.0f * M->sxx, T1 = 3.0f * M->sxy, T2 = 3.0f * M->syy;
                    float h = 1.5f * (M->sxx + M->syy);
                    if (!quadrupole) T0 = T1 = T2 = h = 0.0f;  /* bootstrap pass: monopoles */
                    for (int k = 0; k < cnt; ++k) {
                        float dx = cx - px[k], dy = cy - py[k];
                        float u = dx * dx + dy * dy + eps2;
                        float ri = 1.0f / sqrtf(u), r2 = ri * ri, r3 = ri * r2;
                        float tdx = T0 * dx + T1 * dy, tdy = T1 * dx + T2 * dy;
                        float dtd = dx * tdx + dy * tdy;
                        float coef = M->m + r2 * (2.5f * dtd * r2 - h);
                        ax[k] += r3 * (coef * dx - r2 * tdx);
                        ay[k] += r3 * (coef * dy - r2 * tdy);
                    }
                    entries += 1;
                } else if (last[node] - first[node] + 1 <= bucket) {
                    for (int b = first[node]; b <= last[node]; ++b) {
                        for (int k = 0; k < cnt; ++k) p2p_cpu(sx[b], sy[b], sm[b], px[k], py[k], eps2, &ax[k], &ay[k]);
                        entries += 1;
                    }
                } else {
                    for (int s = 0; s < 4; ++s) {
                        int32_t c = qchild[4 * (size_t)node + s];
                        if (c == INT32_MIN) continue;
                        if (c >= 0) {
                            if (top == cap) {
                                cap *= 2;
                                stack = (int32_t*)realloc(stack, sizeof(int32_t) * (size_t)cap);
                            }
                            stack[top++] = c;
                        } else {
                            int b = ~c;
                            for (int k = 0; k < cnt; ++k) p2p_cpu(sx[b], sy[b], sm[b], px[k], py[k], eps2, &ax[k], &ay[k]);
                            entries += 1;
                        }
                    }
                }
            }
            for (int k = 0; k < cnt; ++k) {
                sax[g0 + k] = G * ax[k];
                say[g0 + k] = G * ay[k];
            }
            total += entries * cnt;
        }
        free(stack);
    }
    free(mom);
    free(ropen2);
    free(qerr);
    return total;
}

/* ------------------------------------------------------------------ shared frontiers
 * The engine's k_frontier (bh_walk.cuh) and the walk's frontier start,
 * restated to check that a group starting from its super-group's frontier
 * accepts exactly the cells, and interacts exactly the bodies, that it would
 * from the root.  Decisions are orc_walk_acc's: group box, then the exact
 * minimum over the group when the box is inconclusive; relative rule
 * qerr <= aa d^4 sqrt(d). */
typedef struct {
    const Mom* mom;
    const float *ropen2, *qerr;
    const int32_t *first, *last, *qchild;
    int bucket;
} WalkCtx;

static int cmp_i32(const void* a, const void* b) {
    int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return x < y ? -1 : (x > y);
}

/* One group's decisions from an initial stack: accepted nodes to acc[],
 * directly interacted bodies to bod[] (both sorted); returns node tests. */
static int64_t group_sets(const WalkCtx* c, const float* px, const float* py, int cnt, float aa,
                          const int32_t* init, int ninit, int32_t** stack, int* cap,
                          int32_t** acc, int* nacc, int* cacc, int32_t** bod, int* nbod,
                          int* cbod) {
    float gx0 = px[0], gx1 = px[0], gy0 = py[0], gy1 = py[0];
    for (int k = 0; k < cnt; ++k) {
        gx0 = fminf(gx0, px[k]);
        gx1 = fmaxf(gx1, px[k]);
        gy0 = fminf(gy0, py[k]);
        gy1 = fmaxf(gy1, py[k]);
    }
    const float gdiag = sqrtf((gx1 - gx0) * (gx1 - gx0) + (gy1 - gy0) * (gy1 - gy0));
    int top = 0;
    int64_t tests = 0;
    for (int q = 0; q < ninit; ++q) (*stack)[top++] = init[q];
#define PUSH(arr, num, capv, val)                                              \
    do {                                                                       \
        if (*(num) == *(capv)) {                                               \
            *(capv) *= 2;                                                      \
            *(arr) = (int32_t*)realloc(*(arr), sizeof(int32_t) * (size_t)*(capv)); \
        }                                                                      \
        (*(arr))[(*(num))++] = (val);                                          \
    } while (0)
    while (top > 0) {
        int32_t node = (*stack)[--top];
        ++tests;
        float cx = c->mom[node].cx, cy = c->mom[node].cy;
        float ddx = fmaxf(fmaxf(gx0 - cx, cx - gx1), 0.0f);
        float ddy = fmaxf(fmaxf(gy0 - cy, cy - gy1), 0.0f);
        float d2 = ddx * ddx + ddy * ddy;
        if (d2 <= c->ropen2[node]) {
            float reach = sqrtf(d2) + gdiag;
            if (reach * reach > c->ropen2[node]) {
                d2 = INFINITY;
                for (int k = 0; k < cnt; ++k) {
                    float dx = px[k] - cx, dy = py[k] - cy;
                    float q = dx * dx + dy * dy;
                    d2 = q < d2 ? q : d2;
                }
            }
        }
        int accept = d2 > c->ropen2[node] && c->qerr[node] <= aa * d2 * d2 * sqrtf(d2);
        if (accept) {
            PUSH(acc, nacc, cacc, node);
        } else if (c->last[node] - c->first[node] + 1 <= c->bucket) {
            for (int b = c->first[node]; b <= c->last[node]; ++b) PUSH(bod, nbod, cbod, b);
        } else {
            for (int s4 = 0; s4 < 4; ++s4) {
                int32_t ch = c->qchild[4 * (size_t)node + s4];
                if (ch == INT32_MIN) continue;
                if (ch >= 0) {
                    if (top == *cap) {
                        *cap *= 2;
                        *stack = (int32_t*)realloc(*stack, sizeof(int32_t) * (size_t)*cap);
                    }
                    (*stack)[top++] = ch;
                } else {
                    PUSH(bod, nbod, cbod, ~ch);
                }
            }
        }
    }
#undef PUSH
    qsort(*acc, (size_t)*nacc, sizeof(int32_t), cmp_i32);
    qsort(*bod, (size_t)*nbod, sizeof(int32_t), cmp_i32);
    return tests;
}

void orc_frontier_check(int n, const float* sx, const float* sy, const float* sm,
                        const uint64_t* skeys, const int32_t* left, const int32_t* right,
                        const int32_t* split, const int32_t* first, const int32_t* last,
                        const int32_t* qchild, const float* box, float theta, float G, int bucket,
                        float alpha, const float* aold, int group, int super, int64_t* stats) {
    for (int k = 0; k < 5; ++k) stats[k] = 0;
    if (n < 2) return;
    Mom* mom = (Mom*)malloc(sizeof(Mom) * (size_t)(n - 1));
    acc_moments(0, left, right, sx, sy, sm, mom);
    float* ropen2 = (float*)malloc(sizeof(float) * (size_t)(n - 1));
    float* qerr = (float*)malloc(sizeof(float) * (size_t)(n - 1));
    open_radii(n, mom, skeys, split, first, box, theta, G, ropen2, qerr);
    const WalkCtx c = {mom, ropen2, qerr, first, last, qchild, bucket};
    const int nsup = (n + super - 1) / super;
    int64_t diff = 0, fnodes = 0, facc = 0, t_root = 0, t_front = 0;
#pragma omp parallel reduction(+ : diff, fnodes, facc, t_root, t_front)
    {
        int cap = 4096, cacc0 = 1024, cbod0 = 1024, cacc1 = 1024, cbod1 = 1024;
        int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
        int32_t* fr = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
        int32_t* frs = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
        int32_t *acc0 = (int32_t*)malloc(4096), *bod0 = (int32_t*)malloc(4096);
        int32_t *acc1 = (int32_t*)malloc(4096), *bod1 = (int32_t*)malloc(4096);
#pragma omp for schedule(dynamic, 1)
        for (int S = 0; S < nsup; ++S) {
            const int s0 = S * super, s1 = s0 + super < n ? s0 + super : n;
            float bx0 = sx[s0], bx1 = sx[s0], by0 = sy[s0], by1 = sy[s0];
            for (int i = s0; i < s1; ++i) {
                bx0 = fminf(bx0, sx[i]);
                bx1 = fmaxf(bx1, sx[i]);
                by0 = fminf(by0, sy[i]);
                by1 = fmaxf(by1, sy[i]);
            }
            /* the frontier: open what every group opens */
            int top = 0, nf = 0;
            frs[top++] = 0;
            while (top > 0) {
                int32_t node = frs[--top];
                float cx = mom[node].cx, cy = mom[node].cy;
                float fx = fmaxf(fabsf(cx - bx0), fabsf(cx - bx1));
                float fy = fmaxf(fabsf(cy - by0), fabsf(cy - by1));
                int open = last[node] - first[node] + 1 > bucket && fx * fx + fy * fy <= ropen2[node];
                for (int s4 = 0; open && s4 < 4; ++s4) {
                    int32_t ch = qchild[4 * (size_t)node + s4];
                    if (ch != INT32_MIN && ch < 0) open = 0;  /* a body child */
                }
                if (open) {
                    for (int s4 = 0; s4 < 4; ++s4) {
                        int32_t ch = qchild[4 * (size_t)node + s4];
                        if (ch >= 0) frs[top++] = ch;
                    }
                } else {
                    fr[nf++] = node;
                }
            }
            /* the smallest group scale of the super-group, 0.1 % low */
            float aa = INFINITY;
            if (aold && alpha > 0.0f) {
                for (int g0 = s0; g0 < s1; g0 += group) {
                    int cnt = s1 - g0 < group ? s1 - g0 : group;
                    float amin = INFINITY, asum = 0.0f;
                    for (int k = 0; k < cnt; ++k) {
                        amin = fminf(amin, aold[g0 + k]);
                        asum += aold[g0 + k];
                    }
                    float a = alpha * fmaxf(amin, 0.1f * asum / (float)cnt);
                    aa = fminf(aa, a);
                }
                aa *= 0.999f;
            }
            /* frontier cells every group accepts */
            int ntest = 0, nacc = 0;
            int32_t* accepted = frs;  /* reuse: the traversal stack is empty now */
            for (int q = 0; q < nf; ++q) {
                int32_t node = fr[q];
                float cx = mom[node].cx, cy = mom[node].cy;
                float ddx = fmaxf(fmaxf(bx0 - cx, cx - bx1), 0.0f);
                float ddy = fmaxf(fmaxf(by0 - cy, cy - by1), 0.0f);
                float d2 = ddx * ddx + ddy * ddy;
                if (d2 > ropen2[node] && qerr[node] <= aa * d2 * d2 * sqrtf(d2))
                    accepted[nacc++] = node;
                else
                    fr[ntest++] = node;
            }
            fnodes += ntest;
            facc += nacc;
            /* each group: root start against frontier start */
            for (int g0 = s0; g0 < s1; g0 += group) {
                int cnt = s1 - g0 < group ? s1 - g0 : group;
                float ga = INFINITY;
                if (aold && alpha > 0.0f) {
                    float amin = INFINITY, amean = 0.0f;
                    for (int k = 0; k < cnt; ++k) {
                        amin = fminf(amin, aold[g0 + k]);
                        amean += aold[g0 + k];
                    }
                    amean /= (float)cnt;
                    ga = alpha * fmaxf(amin, 0.1f * amean);
                }
                int na0 = 0, nb0 = 0, na1 = 0, nb1 = 0;
                int32_t root = 0;
                t_root += group_sets(&c, sx + g0, sy + g0, cnt, ga, &root, 1, &stack, &cap, &acc0,
                                     &na0, &cacc0, &bod0, &nb0, &cbod0);
                t_front += group_sets(&c, sx + g0, sy + g0, cnt, ga, fr, ntest, &stack, &cap,
                                      &acc1, &na1, &cacc1, &bod1, &nb1, &cbod1);
                /* the untested accepted cells join the frontier start's cells */
                if (na1 + nacc > cacc1) {
                    cacc1 = na1 + nacc;
                    acc1 = (int32_t*)realloc(acc1, sizeof(int32_t) * (size_t)cacc1);
                }
                memcpy(acc1 + na1, accepted, sizeof(int32_t) * (size_t)nacc);
                na1 += nacc;
                qsort(acc1, (size_t)na1, sizeof(int32_t), cmp_i32);
                if (na0 != na1 || nb0 != nb1 ||
                    memcmp(acc0, acc1, sizeof(int32_t) * (size_t)na0) != 0 ||
                    memcmp(bod0, bod1, sizeof(int32_t) * (size_t)nb0) != 0)
                    ++diff;
            }
        }
        free(stack);
        free(fr);
        free(frs);
        free(acc0);
        free(bod0);
        free(acc1);
        free(bod1);
    }
    stats[0] = diff;
    stats[1] = fnodes;
    stats[2] = facc;
    stats[3] = t_root;
    stats[4] = t_front;
    free(mom);
    free(ropen2);
    free(qerr);
}

/* ------------------------------------------------------------------ tree invariants
 * The engine's bh_check restated (one system).  debug.cpp:23-174 checks the
 * reference's pointer quadtree on the host: child counts add up (:20-37),
 * every body is a child once (:43-55), child indices in range (:57-83),
 * sorted[] a permutation (:110-146), box ordered (:152-166).  The same
 * statements for a binary radix tree, with every index range-checked. */
unsigned orc_check_tree(int n, const uint64_t* skeys, const int32_t* left, const int32_t* right,
                        const int32_t* parent, const int32_t* leaf_parent, const int32_t* first,
                        const int32_t* last, const float* sm, const float* node_m,
                        const int32_t* id, const float* box) {
    enum { COUNT = 1, CHILD_SUM = 2, CHILD_RANGE = 4, PARENT = 8, KEYS = 16, PERM = 32, BOX = 64,
           MASS = 128 };
    unsigned f = 0;
    unsigned long long psum = 0, leaves = 0;
    if (n == 1) {
        psum = 0;
        leaves = 1;
    }
    for (int i = 0; i < n - 1; ++i) {
        const int a = first[i], b = last[i];
        if (a < 0 || b > n - 1 || a >= b || (a != i && b != i)) f |= COUNT;
        const int ch[2] = {left[i], right[i]};
        int cf[2] = {0, 0}, cl[2] = {0, 0};
        float cm[2] = {0.0f, 0.0f};
        int ok = 1;
        for (int q = 0; q < 2; ++q) {
            const int c = ch[q];
            if (c == INT32_MIN) {
                ok = 0;
            } else if (c < 0) {
                const int body = ~c;
                if (body < 0 || body > n - 1) {
                    ok = 0;
                } else {
                    psum += (unsigned long long)body;
                    leaves += 1;
                    if (leaf_parent[body] != i) f |= PARENT;
                    cf[q] = cl[q] = body;
                    cm[q] = sm[body];
                }
            } else if (c >= n - 1) {
                ok = 0;
            } else {
                if (parent[c] != i) f |= PARENT;
                cf[q] = first[c];
                cl[q] = last[c];
                cm[q] = node_m[c];
            }
        }
        if (!ok) {
            f |= CHILD_RANGE;
        } else {
            if (cf[0] != a || cl[1] != b || cl[0] + 1 != cf[1]) f |= COUNT;
            const float msum = cm[0] + cm[1];
            if (msum != node_m[i]) f |= MASS;
        }
    }
    const unsigned long long nn = (unsigned long long)n;
    if (psum != nn * (nn - 1) / 2 || leaves != nn) f |= CHILD_SUM;
    int* seen = (int*)calloc((size_t)n, sizeof(int));
    for (int j = 0; j < n; ++j) {
        if (j + 1 < n && skeys[j] > skeys[j + 1]) f |= KEYS;
        const int c = id[j];
        if (c < 0 || c >= n)
            f |= PERM;
        else
            seen[c] += 1;
    }
    for (int j = 0; j < n; ++j)
        if (seen[j] != 1) f |= PERM;
    free(seen);
    if (!(box[0] <= box[1]) || !(box[2] <= box[3])) f |= BOX;
    return f;
}

/* ------------------------------------------------------------------ rendering
 * The reference draws the output buffer as one-pixel points through
 * glm::ortho(-25, 25, -25, 25) with colour (1,1,1,0.1) and blend
 * (GL_SRC_ALPHA, GL_ONE) over a (0,0,0,0.5) clear
 * (StellarSolverVisualizer.cpp:4-20, 208-253).  Restated with an exact
 * per-pixel point count, as the engine's bh_render does. */
void orc_render(int n, const float* x, const float* y, int width, int height, float x0, float x1,
                float y0, float y1, unsigned char* rgba) {
    const float sx = (float)width / (x1 - x0), sy = (float)height / (y1 - y0);
    uint32_t* counts = (uint32_t*)calloc((size_t)width * height, sizeof(uint32_t));
    for (int i = 0; i < n; ++i) {
        const float fx = (x[i] - x0) * sx, fy = (y[i] - y0) * sy;
        if (!(fx >= 0.0f) || !(fy >= 0.0f) || !(fx < (float)width) || !(fy < (float)height)) continue;
        const int ix = (int)fx, iy = (int)fy;
        if (ix >= width || iy >= height) continue;
        counts[(size_t)(height - 1 - iy) * width + ix] += 1;
    }
    for (size_t p = 0; p < (size_t)width * height; ++p) {
        const unsigned long long c = counts[p];
        const unsigned v = c >= 10 ? 255u : (unsigned)((255ull * c + 5ull) / 10ull);
        const unsigned a = c >= 50 ? 255u : (unsigned)((255ull * (50ull + c) + 50ull) / 100ull);
        rgba[4 * p] = rgba[4 * p + 1] = rgba[4 * p + 2] = (unsigned char)v;
        rgba[4 * p + 3] = (unsigned char)a;
    }
    free(counts);
}
