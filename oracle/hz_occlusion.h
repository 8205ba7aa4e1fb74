/*
 * hz_occlusion.h -- CPU occlusion-query semantics shared by the oracle and by
 * the Embree/TBB shim used to compile the unmodified reference.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline legs reach this code (through hz_oracle.c or the shim). The
 * product library never includes it.
 *
 * The reference answers its occlusion queries with Embree 4 (not vendored;
 * conda-forge, unpinned): rtcCommitScene builds a BVH over FP32 vertices with
 * RTC_SCENE_FLAG_ROBUST (mo_lradtopo_horayzon.cpp:395-432) and rtcOccluded1
 * reports any hit with t in [tnear, tfar] by setting tfar = -inf
 * (mo_lradtopo_horayzon.cpp:446-460). Embree's own arithmetic is not
 * available here, so this header states the query as published algorithms:
 *
 *   - a linear BVH: 2 x 16-bit Morton codes of the triangle-box centres in the
 *     horizontal (x, y) plane, ties broken by index (Karras, "Maximizing
 *     parallelism in the construction of BVHs, octrees and k-d trees",
 *     HPG 2012), subtrees of <= HZO_LEAF_MAX triangles collapsed into leaves;
 *   - child boxes padded by a scene-relative margin, so that box culling never
 *     removes a triangle the triangle test would report (BVH result ==
 *     brute-force result);
 *   - a slab test with tmax scaled by 1 + 2*gamma(3) (Ize, "Robust BVH ray
 *     traversal", JCGT 2013);
 *   - the watertight ray/triangle test of Woop, Benthin & Wald ("Watertight
 *     ray/triangle intersection", JCGT 2013), including its double-precision
 *     re-evaluation of zero edge functions. Hit iff tnear < t <= tfar.
 *
 * All arithmetic is written in plain IEEE operations; the file must be
 * compiled with -ffp-contract=off so that no multiply-add is fused. The CUDA
 * kernels of the product implement the same triangle test with explicitly
 * rounded intrinsics, which makes hit decisions bit-identical.
 *
 * The typed part at the end of this header is instantiated twice by
 * hz_oracle.c: for float (reference semantics) and for double (the FP64 error
 * oracle).
 */
#ifndef HZ_OCCLUSION_H
#define HZ_OCCLUSION_H

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define HZO_LEAF_MAX 4
#define HZO_STACK 96

typedef struct {
    int64_t node_visits; /* internal-node fetches */
    int64_t tri_tests;   /* triangle tests */
    int64_t overflow;    /* traversal-stack overflows (must stay 0) */
} hzo_counts;

/* Spread the low 16 bits of x to the even bit positions. */
static inline uint32_t hzo_part1by1(uint32_t x) {
    x &= 0x0000FFFFu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

/* Karras 2012 prefix length between sorted keys i and j; -1 outside [0, n). */
static inline int hzo_delta(const uint32_t* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = keys[i], b = keys[j];
    if (a != b) return __builtin_clz(a ^ b);
    return 32 + __builtin_clz((uint32_t)i ^ (uint32_t)j);
}

/* Leaf references are negative: ~(start << 3 | (count - 1)). */
static inline int hzo_leaf_ref(int start, int count) {
    return ~((start << 3) | (count - 1));
}
static inline int hzo_leaf_start(int ref) { return (~ref) >> 3; }
static inline int hzo_leaf_count(int ref) { return ((~ref) & 7) + 1; }

/*
 * Karras 2012, Fig. 4: range and split of internal node i over n sorted keys.
 * Writes the two child references (leaf collapse at HZO_LEAF_MAX) and the
 * range [first, last].
 */
static inline void hzo_karras_node(const uint32_t* keys, int n, int i,
                                   int* child0, int* child1, int* first_out,
                                   int* last_out) {
    int d = (hzo_delta(keys, n, i, i + 1) - hzo_delta(keys, n, i, i - 1)) >= 0
                ? 1 : -1;
    int dmin = hzo_delta(keys, n, i, i - d);
    int lmax = 2;
    while (hzo_delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (hzo_delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = hzo_delta(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (hzo_delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + (d < 0 ? d : 0);
    int first = i < j ? i : j;
    int last = i < j ? j : i;
    int nl = gamma - first + 1;
    int nr = last - gamma;
    *child0 = nl <= HZO_LEAF_MAX ? hzo_leaf_ref(first, nl) : gamma;
    *child1 = nr <= HZO_LEAF_MAX ? hzo_leaf_ref(gamma + 1, nr) : gamma + 1;
    *first_out = first;
    *last_out = last;
}

static int hzo_cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return (x > y) - (x < y);
}

#endif /* HZ_OCCLUSION_H */

/* ------------------------------------------------------------------------- */
/* Typed part: define HZO_REAL (float|double) and HZO_SFX before including.  */
/* ------------------------------------------------------------------------- */
#if defined(HZO_REAL) && defined(HZO_SFX)

#define HZO_CAT2(a, b) a##b
#define HZO_CAT(a, b) HZO_CAT2(a, b)
#define HZO_T(name) HZO_CAT(name, HZO_SFX)

typedef struct {
    int n_tri;
    int n_node;          /* internal nodes (n_tri - 1, some unused) */
    int root;            /* root reference (>= 0 node, < 0 leaf, or INT32_MIN empty) */
    HZO_REAL* box;       /* n_node * 12: child0 lo/hi xyz, child1 lo/hi xyz */
    int* child;          /* n_node * 2 */
    HZO_REAL* tri;       /* n_tri * 9: v0, v1, v2 in sorted order */
    int* tri_id;         /* original triangle index per sorted slot */
    HZO_REAL pad;        /* box margin */
} HZO_T(hzo_bvh_);

typedef struct {
    HZO_REAL o[3];
    HZO_REAL d[3];
    HZO_REAL inv[3];
    int kx, ky, kz;
    HZO_REAL Sx, Sy, Sz;
    HZO_REAL tnear, tfar;
} HZO_T(hzo_ray_);

static void HZO_T(hzo_bvh_free_)(HZO_T(hzo_bvh_)* b) {
    free(b->box); free(b->child); free(b->tri); free(b->tri_id);
    memset(b, 0, sizeof(*b));
}

/* Union of the (sorted) triangles [start, start + count) into lo/hi. */
static void HZO_T(hzo_leaf_box_)(const HZO_T(hzo_bvh_)* b, int start, int count,
                                 HZO_REAL* lo, HZO_REAL* hi) {
    for (int k = 0; k < 3; k++) { lo[k] = INFINITY; hi[k] = -INFINITY; }
    for (int t = start; t < start + count; t++)
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++) {
                HZO_REAL c = b->tri[9 * t + 3 * v + k];
                if (c < lo[k]) lo[k] = c;
                if (c > hi[k]) hi[k] = c;
            }
}

/* Post-order refit: fills the child boxes of node `ref`, returns its box. */
static void HZO_T(hzo_refit_)(HZO_T(hzo_bvh_)* b, int ref, HZO_REAL* lo,
                              HZO_REAL* hi) {
    if (ref < 0) {
        HZO_T(hzo_leaf_box_)(b, hzo_leaf_start(ref), hzo_leaf_count(ref), lo, hi);
        return;
    }
    HZO_REAL l0[3], h0[3], l1[3], h1[3];
    HZO_T(hzo_refit_)(b, b->child[2 * ref], l0, h0);
    HZO_T(hzo_refit_)(b, b->child[2 * ref + 1], l1, h1);
    HZO_REAL* bx = b->box + 12 * (size_t)ref;
    for (int k = 0; k < 3; k++) {
        bx[k] = l0[k] - b->pad;
        bx[3 + k] = h0[k] + b->pad;
        bx[6 + k] = l1[k] - b->pad;
        bx[9 + k] = h1[k] + b->pad;
        lo[k] = l0[k] < l1[k] ? l0[k] : l1[k];
        hi[k] = h0[k] > h1[k] ? h0[k] : h1[k];
    }
}

/*
 * Build the LBVH over n_tri triangles. `vert` holds xyz per mesh vertex in
 * HZO_REAL, `vot` three vertex indices per triangle. Returns 0 on success.
 */
static int HZO_T(hzo_bvh_build_)(HZO_T(hzo_bvh_)* b, const HZO_REAL* vert,
                                 const int* vot, int n_tri) {
    memset(b, 0, sizeof(*b));
    b->n_tri = n_tri;
    b->root = INT32_MIN;
    if (n_tri <= 0) return 0;
    b->tri = (HZO_REAL*)malloc(sizeof(HZO_REAL) * 9 * (size_t)n_tri);
    b->tri_id = (int*)malloc(sizeof(int) * (size_t)n_tri);
    HZO_REAL* cen = (HZO_REAL*)malloc(sizeof(HZO_REAL) * 2 * (size_t)n_tri);
    uint64_t* kv = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n_tri);
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n_tri);
    if (!b->tri || !b->tri_id || !cen || !kv || !keys) {
        free(cen); free(kv); free(keys); HZO_T(hzo_bvh_free_)(b);
        return -1;
    }
    HZO_REAL cmin[2] = {INFINITY, INFINITY}, cmax[2] = {-INFINITY, -INFINITY};
    HZO_REAL maxabs = 0;
    for (int t = 0; t < n_tri; t++) {
        HZO_REAL lo[3] = {INFINITY, INFINITY, INFINITY};
        HZO_REAL hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++) {
                HZO_REAL c = vert[3 * (size_t)vot[3 * (size_t)t + v] + k];
                if (c < lo[k]) lo[k] = c;
                if (c > hi[k]) hi[k] = c;
                HZO_REAL a = c < 0 ? -c : c;
                if (a > maxabs) maxabs = a;
            }
        for (int k = 0; k < 2; k++) {
            HZO_REAL c = (lo[k] + hi[k]) * (HZO_REAL)0.5;
            cen[2 * (size_t)t + k] = c;
            if (c < cmin[k]) cmin[k] = c;
            if (c > cmax[k]) cmax[k] = c;
        }
    }
    HZO_REAL scale[2];
    for (int k = 0; k < 2; k++) {
        HZO_REAL ext = cmax[k] - cmin[k];
        scale[k] = ext > 0 ? (HZO_REAL)65535.0 / ext : (HZO_REAL)0.0;
    }
    for (int t = 0; t < n_tri; t++) {
        uint32_t q[2];
        for (int k = 0; k < 2; k++) {
            HZO_REAL f = (cen[2 * (size_t)t + k] - cmin[k]) * scale[k];
            q[k] = f <= 0 ? 0u : (f >= (HZO_REAL)65535.0 ? 65535u : (uint32_t)f);
        }
        uint32_t key = hzo_part1by1(q[0]) | (hzo_part1by1(q[1]) << 1);
        kv[t] = ((uint64_t)key << 32) | (uint32_t)t;
    }
    qsort(kv, (size_t)n_tri, sizeof(uint64_t), hzo_cmp_u64);
    for (int s = 0; s < n_tri; s++) {
        keys[s] = (uint32_t)(kv[s] >> 32);
        int t = (int)(kv[s] & 0xFFFFFFFFu);
        b->tri_id[s] = t;
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++)
                b->tri[9 * (size_t)s + 3 * v + k] =
                    vert[3 * (size_t)vot[3 * (size_t)t + v] + k];
    }
    free(cen); free(kv);
    /* Margin: 2^-20 of the largest coordinate (float), 2^-40 (double). */
    b->pad = sizeof(HZO_REAL) == 4 ? maxabs * (HZO_REAL)9.5367431640625e-07
                                   : maxabs * (HZO_REAL)9.094947017729282e-13;
    if (n_tri <= HZO_LEAF_MAX) {
        /* Root is a single node whose second child is empty. */
        b->n_node = 1;
        b->box = (HZO_REAL*)malloc(sizeof(HZO_REAL) * 12);
        b->child = (int*)malloc(sizeof(int) * 2);
        b->child[0] = hzo_leaf_ref(0, n_tri);
        b->child[1] = INT32_MIN;
        HZO_REAL lo[3], hi[3];
        HZO_T(hzo_leaf_box_)(b, 0, n_tri, lo, hi);
        for (int k = 0; k < 3; k++) {
            b->box[k] = lo[k] - b->pad; b->box[3 + k] = hi[k] + b->pad;
            b->box[6 + k] = INFINITY; b->box[9 + k] = -INFINITY;
        }
        b->root = 0;
        free(keys);
        return 0;
    }
    b->n_node = n_tri - 1;
    b->box = (HZO_REAL*)malloc(sizeof(HZO_REAL) * 12 * (size_t)b->n_node);
    b->child = (int*)malloc(sizeof(int) * 2 * (size_t)b->n_node);
    if (!b->box || !b->child) { free(keys); HZO_T(hzo_bvh_free_)(b); return -1; }
    for (int i = 0; i < b->n_node; i++) {
        int f, l;
        hzo_karras_node(keys, n_tri, i, &b->child[2 * i], &b->child[2 * i + 1],
                        &f, &l);
    }
    free(keys);
    b->root = 0;
    HZO_REAL lo[3], hi[3];
    HZO_T(hzo_refit_)(b, 0, lo, hi);
    return 0;
}

static void HZO_T(hzo_ray_setup_)(HZO_T(hzo_ray_)* r, const HZO_REAL* o,
                                  const HZO_REAL* d, HZO_REAL tnear,
                                  HZO_REAL tfar) {
    for (int k = 0; k < 3; k++) {
        r->o[k] = o[k];
        r->d[k] = d[k];
        r->inv[k] = (HZO_REAL)1.0 / d[k];
    }
    HZO_REAL ax = fabs(d[0]), ay = fabs(d[1]), az = fabs(d[2]);
    int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0) { int tmp = kx; kx = ky; ky = tmp; }
    r->kx = kx; r->ky = ky; r->kz = kz;
    r->Sx = d[kx] / d[kz];
    r->Sy = d[ky] / d[kz];
    r->Sz = (HZO_REAL)1.0 / d[kz];
    r->tnear = tnear;
    r->tfar = tfar;
}

/* Woop, Benthin & Wald 2013 watertight test; 1 = hit with tnear < t <= tfar. */
static inline int HZO_T(hzo_tri_hit_)(const HZO_T(hzo_ray_)* r,
                                      const HZO_REAL* v) {
    const int kx = r->kx, ky = r->ky, kz = r->kz;
    HZO_REAL A[3], B[3], C[3];
    for (int k = 0; k < 3; k++) {
        A[k] = v[k] - r->o[k];
        B[k] = v[3 + k] - r->o[k];
        C[k] = v[6 + k] - r->o[k];
    }
    HZO_REAL Ax = A[kx] - r->Sx * A[kz];
    HZO_REAL Ay = A[ky] - r->Sy * A[kz];
    HZO_REAL Bx = B[kx] - r->Sx * B[kz];
    HZO_REAL By = B[ky] - r->Sy * B[kz];
    HZO_REAL Cx = C[kx] - r->Sx * C[kz];
    HZO_REAL Cy = C[ky] - r->Sy * C[kz];
    HZO_REAL U = Cx * By - Cy * Bx;
    HZO_REAL V = Ax * Cy - Ay * Cx;
    HZO_REAL W = Bx * Ay - By * Ax;
    if (sizeof(HZO_REAL) == 4 && (U == 0 || V == 0 || W == 0)) {
        U = (HZO_REAL)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (HZO_REAL)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (HZO_REAL)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return 0;
    HZO_REAL det = U + V + W;
    if (det == 0) return 0;
    HZO_REAL Az = r->Sz * A[kz];
    HZO_REAL Bz = r->Sz * B[kz];
    HZO_REAL Cz = r->Sz * C[kz];
    HZO_REAL T = U * Az + V * Bz + W * Cz;
    if (det > 0) return T > r->tnear * det && T <= r->tfar * det;
    return T < r->tnear * det && T >= r->tfar * det;
}

/* Conservative slab test against one (padded) box; 1 = may contain a hit. */
static inline int HZO_T(hzo_box_hit_)(const HZO_T(hzo_ray_)* r,
                                      const HZO_REAL* lo, const HZO_REAL* hi,
                                      HZO_REAL* tentry) {
    const HZO_REAL g3 = sizeof(HZO_REAL) == 4
                            ? (HZO_REAL)(1.0 + 2.0 * 3.0 * 5.9604644775390625e-08 /
                                                   (1.0 - 3.0 * 5.9604644775390625e-08))
                            : (HZO_REAL)(1.0 + 2.0 * 3.0 * 1.1102230246251565e-16 /
                                                   (1.0 - 3.0 * 1.1102230246251565e-16));
    HZO_REAL tmin = r->tnear, tmax = r->tfar;
    for (int k = 0; k < 3; k++) {
        HZO_REAL t0 = (lo[k] - r->o[k]) * r->inv[k];
        HZO_REAL t1 = (hi[k] - r->o[k]) * r->inv[k];
        HZO_REAL tn = fmin(t0, t1), tf = fmax(t0, t1);
        tf = tf * g3;
        tmin = fmax(tmin, tn);
        tmax = fmin(tmax, tf);
    }
    *tentry = tmin;
    return tmin <= tmax;
}

/* Any-hit query. Returns 1 on a hit; counts node and triangle work in c. */
static int HZO_T(hzo_occluded_)(const HZO_T(hzo_bvh_)* b,
                                const HZO_T(hzo_ray_)* r, hzo_counts* c) {
    if (b->root == INT32_MIN) return 0;
    int stack[HZO_STACK];
    int sp = 0;
    int ref = b->root;
    for (;;) {
        if (ref < 0) {
            int s = hzo_leaf_start(ref), n = hzo_leaf_count(ref);
            for (int t = s; t < s + n; t++) {
                c->tri_tests++;
                if (HZO_T(hzo_tri_hit_)(r, b->tri + 9 * (size_t)t)) return 1;
            }
        } else {
            c->node_visits++;
            const HZO_REAL* bx = b->box + 12 * (size_t)ref;
            HZO_REAL t0, t1;
            int h0 = HZO_T(hzo_box_hit_)(r, bx, bx + 3, &t0);
            int h1 = HZO_T(hzo_box_hit_)(r, bx + 6, bx + 9, &t1);
            int c0 = b->child[2 * ref], c1 = b->child[2 * ref + 1];
            if (c1 == INT32_MIN) h1 = 0;
            if (h0 && h1) {
                int near_ref = t0 <= t1 ? c0 : c1;
                int far_ref = t0 <= t1 ? c1 : c0;
                if (sp >= HZO_STACK) { c->overflow++; return 1; }
                stack[sp++] = far_ref;
                ref = near_ref;
                continue;
            }
            if (h0) { ref = c0; continue; }
            if (h1) { ref = c1; continue; }
        }
        if (sp == 0) return 0;
        ref = stack[--sp];
    }
}

/* Brute-force any-hit over every triangle (tiny meshes; checks the BVH). */
static int HZO_T(hzo_occluded_brute_)(const HZO_T(hzo_bvh_)* b,
                                      const HZO_T(hzo_ray_)* r, hzo_counts* c) {
    for (int t = 0; t < b->n_tri; t++) {
        c->tri_tests++;
        if (HZO_T(hzo_tri_hit_)(r, b->tri + 9 * (size_t)t)) return 1;
    }
    return 0;
}

#undef HZO_T
#undef HZO_CAT
#undef HZO_CAT2
#endif /* HZO_REAL && HZO_SFX */
