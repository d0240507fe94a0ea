/*
 * rtoracle.c -- CPU restatement of RAPTor's ray-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA core is compared against,
 * never part of the product.  Compile with -ffp-contract=off (no FMA contraction) so the
 * results are the reference's IEEE binary32 results on any host.
 *
 * Reference paths below are relative to the RAPTor project root.
 */
#define _POSIX_C_SOURCE 200809L
#include "rtoracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* Constants (common/common.cc:14-17). */
#define RO_EPSILON 1.0e-3f
#define RO_FP_DELTA 32.0f
#define RO_FP_DELTA_SMALL 1.0e-4f
#define RO_MAX_DIST FLT_MAX
/* Traversal stack height (common/common.h:63-64). */
#define RO_MAX_STACK 100
#define RO_LEAF_SIZE 4

typedef struct { float x, y, z; } v3;

static inline v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 vdivs(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline v3 vneg(v3 a) { return mk(-a.x, -a.y, -a.z); }
/* dot_product / cross_product (common/point_t.h:498-525), left to right. */
static inline float vdot(v3 a, v3 b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }
static inline v3 vcross(v3 a, v3 b)
{
    return mk((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
/* std::min / std::max semantics: min(a,b) = (b < a) ? b : a. */
static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline float smax(float a, float b) { return (a < b) ? b : a; }
static inline v3 vmin(v3 a, v3 b) { return mk(smin(a.x, b.x), smin(a.y, b.y), smin(a.z, b.z)); }
static inline v3 vmax(v3 a, v3 b) { return mk(smax(a.x, b.x), smax(a.y, b.y), smax(a.z, b.z)); }
/* magnitude (point_t.h:357) and normalise with EXACT_NORMALISE (point_t.h:571-585). */
static inline float vmag(v3 a) { return sqrtf(((a.x * a.x) + (a.y * a.y)) + (a.z * a.z)); }
static inline v3 vnorm(v3 a)
{
    const float d = sqrtf(((a.x * a.x) + (a.y * a.y)) + (a.z * a.z));
    return mk(a.x / d, a.y / d, a.z / d);
}
static inline v3 ld3(const float *p) { return mk(p[0], p[1], p[2]); }

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* float -> int32 truncation with the x86 cvttss2si result for NaN and
 * out-of-range inputs (the integer-indefinite value), so hosts agree. */
static inline int32_t cvtt(float f)
{
    if (!(f > -2147483904.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int32_t)f;
}

/* ---------------------------------------------------------------- Morton */

/* split_by_three + morton_code (common/simd.h:798-825). */
static inline uint32_t split3(uint32_t a)
{
    a |= (a << 16); a &= 0x030000FFu;
    a |= (a << 8);  a &= 0x0300F00Fu;
    a |= (a << 4);  a &= 0x030C30C3u;
    a |= (a << 2);  a &= 0x09249249u;
    return a;
}

int32_t ro_morton_code(float x, float y, float z, float x_mul, float y_mul, float z_mul)
{
    const uint32_t xi = split3((uint32_t)cvtt(x * x_mul));
    const uint32_t yi = split3((uint32_t)cvtt(y * y_mul));
    const uint32_t zi = split3((uint32_t)cvtt(z * z_mul));
    return (int32_t)(xi | (yi << 1) | (zi << 2));
}

/* ----------------------------------------------------------------- Scene */

typedef struct ro_node {
    v3 lo, hi;          /* bvh_node::_low / _high (bvh_node.h:294-311) */
    int32_t a, b;       /* leaf: [a, b) into indirect; inner: left, right */
    int32_t leaf;
} ro_node;

struct ro_scene {
    int32_t ntris;
    v3 *va, *vb, *vc;   /* triangle vertices (triangle.h:108-110) */
    v3 *n;              /* face normal (triangle.h:170-175) */
    v3 *ta, *tb, *tc;   /* per-vertex attribute (triangle vnt[3..5]) or NULL */
    uint32_t *flags;
    ro_node *nodes;
    int32_t nnodes, root;
    int32_t *indirect;  /* primitive_store::_indirect */
    int32_t *mat;       /* material index per triangle, or NULL (all 0) */
    float *cn;          /* corner normals, 9 floats per triangle, or NULL (x of a = FLT_MAX: none) */
};

ro_scene *ro_scene_create(const float *verts, int32_t nverts, const int32_t *tris, int32_t ntris,
                          const float *vattr, const uint32_t *flags)
{
    if (ntris < 0 || nverts < 0) return NULL;
    ro_scene *s = (ro_scene *)calloc(1, sizeof(ro_scene));
    if (!s) return NULL;
    s->ntris = ntris;
    const size_t nt = (size_t)(ntris > 0 ? ntris : 1);
    s->va = (v3 *)malloc(nt * sizeof(v3));
    s->vb = (v3 *)malloc(nt * sizeof(v3));
    s->vc = (v3 *)malloc(nt * sizeof(v3));
    s->n = (v3 *)malloc(nt * sizeof(v3));
    s->flags = (uint32_t *)calloc(nt, sizeof(uint32_t));
    if (vattr) {
        s->ta = (v3 *)malloc(nt * sizeof(v3));
        s->tb = (v3 *)malloc(nt * sizeof(v3));
        s->tc = (v3 *)malloc(nt * sizeof(v3));
    }
    for (int32_t i = 0; i < ntris; ++i) {
        const int32_t ia = tris[3 * i], ib = tris[3 * i + 1], ic = tris[3 * i + 2];
        if (ia < 0 || ib < 0 || ic < 0 || ia >= nverts || ib >= nverts || ic >= nverts) {
            ro_scene_destroy(s);
            return NULL;
        }
        s->va[i] = ld3(verts + 3 * (size_t)ia);
        s->vb[i] = ld3(verts + 3 * (size_t)ib);
        s->vc[i] = ld3(verts + 3 * (size_t)ic);
        /* triangle::triangle normal (triangle.h:171-175): (b-a) x (c-a), normalised */
        s->n[i] = vnorm(vcross(vsub(s->vb[i], s->va[i]), vsub(s->vc[i], s->va[i])));
        if (vattr) {
            s->ta[i] = ld3(vattr + 3 * (size_t)ia);
            s->tb[i] = ld3(vattr + 3 * (size_t)ib);
            s->tc[i] = ld3(vattr + 3 * (size_t)ic);
        }
        if (flags) s->flags[i] = flags[i];
    }
    return s;
}

void ro_scene_destroy(ro_scene *s)
{
    if (s) free(s->mat);
    if (s) free(s->cn);
    if (!s) return;
    free(s->va); free(s->vb); free(s->vc); free(s->n);
    free(s->ta); free(s->tb); free(s->tc); free(s->flags);
    free(s->nodes); free(s->indirect);
    free(s);
}

int32_t ro_scene_node_count(const ro_scene *s) { return s ? s->nnodes : 0; }

/* -------------------------------------------------------------- Builder */

typedef struct {
    ro_scene *s;
    const uint32_t *codes;  /* Morton code per sorted position */
    v3 *plo, *phi;          /* primitive bounds, original order */
    int32_t next;
} build_ctx;

static inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

/* Top-down split of the Morton-sorted range [b, e) at the highest differing
 * bit (stand-in for the reference's AAC clustering, see the file header). */
static int32_t build_range(build_ctx *c, int32_t b, int32_t e)
{
    const int32_t me = c->next++;
    ro_node *nd = &c->s->nodes[me];
    v3 lo = mk(RO_MAX_DIST, RO_MAX_DIST, RO_MAX_DIST), hi = mk(-RO_MAX_DIST, -RO_MAX_DIST, -RO_MAX_DIST);
    for (int32_t i = b; i < e; ++i) {
        const int32_t p = c->s->indirect[i];
        lo = vmin(lo, c->plo[p]);
        hi = vmax(hi, c->phi[p]);
    }
    nd->lo = lo; nd->hi = hi;
    if (e - b <= RO_LEAF_SIZE) {
        nd->a = b; nd->b = e; nd->leaf = 1;
        return me;
    }
    int32_t split;
    const uint32_t cf = c->codes[b], cl = c->codes[e - 1];
    if (cf == cl) {
        split = (b + e) >> 1;
    } else {
        const int common = clz32(cf ^ cl);
        split = b;
        int32_t step = e - 1 - b;
        do {   /* binary search for the last code sharing more than `common` bits */
            step = (step + 1) >> 1;
            const int32_t ns = split + step;
            if (ns < e - 1 && clz32(cf ^ c->codes[ns]) > common) split = ns;
        } while (step > 1);
        split += 1;
    }
    const int32_t l = build_range(c, b, split);
    const int32_t r = build_range(c, split, e);
    nd = &c->s->nodes[me];
    nd->a = l; nd->b = r; nd->leaf = 0;
    return me;
}

double ro_scene_build(ro_scene *s)
{
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    if (!s) return -1.0;
    const int32_t n = s->ntris;
    free(s->nodes); free(s->indirect);
    s->nodes = (ro_node *)calloc((size_t)(n > 0 ? 2 * n : 1), sizeof(ro_node));
    s->indirect = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    if (!s->nodes || !s->indirect) return -1.0;
    if (n == 0) {
        s->nnodes = 1; s->root = 0;
        s->nodes[0].lo = mk(RO_MAX_DIST, RO_MAX_DIST, RO_MAX_DIST);
        s->nodes[0].hi = mk(-RO_MAX_DIST, -RO_MAX_DIST, -RO_MAX_DIST);
        s->nodes[0].leaf = 1;
        return 0.0;
    }
    const size_t nn = (size_t)(uint32_t)n;
    v3 *plo = (v3 *)malloc(nn * sizeof(v3));
    v3 *phi = (v3 *)malloc(nn * sizeof(v3));
    uint32_t *code = (uint32_t *)malloc(nn * sizeof(uint32_t));
    uint32_t *code2 = (uint32_t *)malloc(nn * sizeof(uint32_t));
    int32_t *idx2 = (int32_t *)malloc(nn * sizeof(int32_t));
    if (!plo || !phi || !code || !code2 || !idx2) {
        free(plo); free(phi); free(code); free(code2); free(idx2);
        return -1.0;
    }
    /* Primitive and scene bounds (bvh_builder.cc:30-42, triangle.h:56-57). */
    v3 sb = mk(RO_MAX_DIST, RO_MAX_DIST, RO_MAX_DIST), st = mk(-RO_MAX_DIST, -RO_MAX_DIST, -RO_MAX_DIST);
    for (int32_t i = 0; i < n; ++i) {
        plo[i] = vmin(s->va[i], vmin(s->vb[i], s->vc[i]));
        phi[i] = vmax(s->va[i], vmax(s->vb[i], s->vc[i]));
        sb = vmin(sb, plo[i]);
        st = vmax(st, phi[i]);
    }
    /* Morton codes of box centres (bvh_builder.cc:45-106). */
    const v3 sw = vsub(st, sb);
    const v3 width = vmul(sw, 1.00001f / 1024.0f);
    const v3 winv = mk(1.0f / width.x, 1.0f / width.y, 1.0f / width.z);
    for (int32_t i = 0; i < n; ++i) {
        const v3 t = vsub(vmul(vadd(phi[i], plo[i]), 0.5f), sb);
        code[i] = (uint32_t)ro_morton_code(t.x, t.y, t.z, winv.x, winv.y, winv.z);
        s->indirect[i] = i;
    }
    /* Three stable 10-bit counting passes, low digit first (bvh_builder.cc:108-158);
     * the 32-bit code is masked per digit so garbage high bits stay in range. */
    for (int pass = 0; pass < 3; ++pass) {
        uint32_t hist[1025];
        memset(hist, 0, sizeof(hist));
        const int sh = 10 * pass;
        for (int32_t i = 0; i < n; ++i) hist[((code[i] >> sh) & 0x3ffu) + 1]++;
        for (int k = 0; k < 1024; ++k) hist[k + 1] += hist[k];
        for (int32_t i = 0; i < n; ++i) {
            const uint32_t d = (code[i] >> sh) & 0x3ffu;
            const uint32_t pos = hist[d]++;
            code2[pos] = code[i];
            idx2[pos] = s->indirect[i];
        }
        memcpy(code, code2, nn * sizeof(uint32_t));
        memcpy(s->indirect, idx2, nn * sizeof(int32_t));
    }
    build_ctx c = {s, code, plo, phi, 0};
    s->root = build_range(&c, 0, n);
    s->nnodes = c.next;
    free(plo); free(phi); free(code); free(code2); free(idx2);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* ------------------------------------------------------------ Traversal */

typedef struct { v3 o, d; } ro_ray;
typedef struct { float u, v, d; } ro_hit;

/* triangle::is_intersecting (triangle.h:190-235): Moller-Trumbore with
 * e1 = c - a, e2 = b - a; u weighs c, v weighs b.  Leaves h untouched when
 * t <= EPSILON, sets d = MAX_DIST on any other rejection. */
static inline void isect(const ro_scene *s, int32_t i, const ro_ray *r, ro_hit *h)
{
    const v3 a = s->va[i];
    const v3 e1 = vsub(s->vc[i], a);
    const v3 e2 = vsub(s->vb[i], a);
    const v3 P = vcross(r->d, e2);
    const float det = vdot(e1, P);
    if (det > -0.000001f && det < 0.000001f) { h->d = RO_MAX_DIST; return; }
    const float inv_det = 1.0f / det;
    const v3 T = vsub(r->o, a);
    const float u = vdot(T, P) * inv_det;
    if (u < 0.0f) { h->d = RO_MAX_DIST; return; }
    const v3 Q = vcross(T, e1);
    const float v = vdot(r->d, Q) * inv_det;
    if ((v < 0.0f) || ((u + v) > 1.0f)) { h->d = RO_MAX_DIST; return; }
    const float t = vdot(e2, Q) * inv_det;
    if (t > RO_EPSILON) { h->d = t; h->u = u; h->v = v; }
}

/* bvh_node::intersection_distance (bvh_node.h:61-98). */
static inline float slab(const ro_node *nd, const ro_ray *r, v3 ird)
{
    v3 ld = mk((nd->lo.x - r->o.x) * ird.x, (nd->lo.y - r->o.y) * ird.y, (nd->lo.z - r->o.z) * ird.z);
    v3 hd = mk((nd->hi.x - r->o.x) * ird.x, (nd->hi.y - r->o.y) * ird.y, (nd->hi.z - r->o.z) * ird.z);
    float tmp;
    if (ld.x > hd.x) { tmp = ld.x; ld.x = hd.x; hd.x = tmp; }
    if (ld.y > hd.y) { tmp = ld.y; ld.y = hd.y; hd.y = tmp; }
    if (ld.z > hd.z) { tmp = ld.z; ld.z = hd.z; hd.z = tmp; }
    const float exit_t = smin(smin(hd.x, hd.y), hd.z);
    const float enter_t = smax(smax(ld.x, ld.y), ld.z);
    if (smax(0.0f, enter_t) > exit_t) return RO_MAX_DIST;
    return enter_t;
}

typedef struct { float t_min; int32_t idx; } stack_el;

/* bvh::find_leaf_node (bvh.cc:586-647).  Returns 1 with *cur at a leaf, or 0
 * when both children lie beyond t_max + 100 EPSILON. */
static inline int find_leaf(const ro_scene *s, const ro_ray *r, v3 ird, float t_max, int32_t *cur,
                            stack_el *stack, int *sp, int *overflow)
{
    int32_t idx = *cur;
    for (;;) {
        const ro_node *nd = &s->nodes[idx];
        if (nd->leaf) { *cur = idx; return 1; }
        int32_t near_idx = nd->a, far_idx = nd->b;
        float near_d = slab(&s->nodes[near_idx], r, ird);
        float far_d = slab(&s->nodes[far_idx], r, ird);
        if (near_d > far_d) {
            int32_t ti = near_idx; near_idx = far_idx; far_idx = ti;
            float tf = near_d; near_d = far_d; far_d = tf;
        }
        if (near_d >= (t_max + (100.0f * RO_EPSILON))) return 0;
        if (far_d >= (t_max + (100.0f * RO_EPSILON))) {
            idx = near_idx;
        } else {
            if (*sp + 1 >= RO_MAX_STACK) { *overflow = 1; return 0; }
            ++*sp;
            stack[*sp].idx = far_idx;
            stack[*sp].t_min = far_d;
            idx = near_idx;
        }
    }
}

/* bvh::find_nearest_object (bvh.cc:649-709) with test_leaf_node_nearest
 * (bvh_node.h:152-168).  Returns the original triangle id or -1. */
static int32_t closest(const ro_scene *s, const ro_ray *r, ro_hit *out)
{
    ro_hit best = {0.0f, 0.0f, RO_MAX_DIST};
    const v3 ird = mk(1.0f / r->d.x, 1.0f / r->d.y, 1.0f / r->d.z);
    if (s->ntris == 0 || slab(&s->nodes[s->root], r, ird) == RO_MAX_DIST) { *out = best; return -1; }
    stack_el stack[RO_MAX_STACK];
    int sp = 0, overflow = 0;
    stack[0].idx = s->root; stack[0].t_min = RO_MAX_DIST;
    int32_t cur = s->root;
    int32_t hit_obj = -1;
    for (;;) {
        if (find_leaf(s, r, ird, best.d, &cur, stack, &sp, &overflow)) {
            const ro_node *nd = &s->nodes[cur];
            for (int32_t i = nd->a; i < nd->b; ++i) {
                ro_hit h = {0.0f, 0.0f, best.d};
                isect(s, s->indirect[i], r, &h);
                if (h.d < best.d) { best = h; hit_obj = s->indirect[i]; }
            }
        }
        if (overflow) break;
        float tmin;
        do {
            if (sp == 0) { *out = best; return hit_obj; }
            cur = stack[sp].idx;
            tmin = stack[sp].t_min;
            --sp;
        } while (tmin > (best.d + (100.0f * RO_EPSILON)));
    }
    *out = best;
    return hit_obj;
}

/* bvh::found_nearer_object (bvh.cc:711-759) with test_leaf_node_nearer
 * (bvh_node.h:170-190): skips light and transparent triangles. */
static int nearer(const ro_scene *s, const ro_ray *r, float t)
{
    if (s->ntris == 0) return 0;
    const v3 ird = mk(1.0f / r->d.x, 1.0f / r->d.y, 1.0f / r->d.z);
    stack_el stack[RO_MAX_STACK];
    int sp = 0, overflow = 0;
    stack[0].idx = s->root; stack[0].t_min = RO_MAX_DIST;
    int32_t cur = s->root;
    for (;;) {
        if (find_leaf(s, r, ird, t, &cur, stack, &sp, &overflow)) {
            const ro_node *nd = &s->nodes[cur];
            for (int32_t i = nd->a; i < nd->b; ++i) {
                const int32_t p = s->indirect[i];
                if (s->flags[p] & (RO_TRI_LIGHT | RO_TRI_TRANSPARENT)) continue;
                ro_hit h = {0.0f, 0.0f, t};
                isect(s, p, r, &h);
                if (h.d < t) return 1;
            }
        }
        if (overflow || sp == 0) return 0;
        cur = stack[sp].idx;
        --sp;
    }
}

int32_t ro_trace_closest(const ro_scene *s, const float *ogn, const float *dir, int32_t n,
                         int32_t *id, float *t, float *u, float *v)
{
    if (!s || !s->nodes) return -1;
    for (int32_t i = 0; i < n; ++i) {
        ro_ray r = {ld3(ogn + 3 * (size_t)i), ld3(dir + 3 * (size_t)i)};
        ro_hit h;
        id[i] = closest(s, &r, &h);
        t[i] = h.d;
        if (u) u[i] = h.u;
        if (v) v[i] = h.v;
    }
    return 0;
}

int32_t ro_trace_any(const ro_scene *s, const float *ogn, const float *dir, const float *tmax,
                     int32_t n, uint8_t *occluded)
{
    if (!s || !s->nodes) return -1;
    for (int32_t i = 0; i < n; ++i) {
        ro_ray r = {ld3(ogn + 3 * (size_t)i), ld3(dir + 3 * (size_t)i)};
        occluded[i] = (uint8_t)nearer(s, &r, tmax[i]);
    }
    return 0;
}

/* --------------------------------------------------------------- Camera */

typedef struct {
    v3 c, X, Y, Z;
    float x_m, y_m, x_inc, y_inc, t;
} cam_state;

/* base_camera axes go through quaternion_t::rotate with the identity
 * orientation (sdl_wrappers/base_camera.h, common/quaternion_t.h:166-169);
 * restated literally so signed zeros come out as in the reference. */
static v3 identity_rotate(v3 p)
{
    const float qw = 1.0f, qx = 0.0f, qy = 0.0f, qz = 0.0f;
    const v3 c1 = mk((qy * p.z) - (qz * p.y), (qz * p.x) - (qx * p.z), (qx * p.y) - (qy * p.x));
    const v3 c2 = mk((qy * c1.z) - (qz * c1.y), (qz * c1.x) - (qx * c1.z), (qx * c1.y) - (qy * c1.x));
    const v3 a = mk(2.0f * c2.x, 2.0f * c2.y, 2.0f * c2.z);
    const float w2 = 2.0f * qw;
    const v3 b = mk(w2 * c1.x, w2 * c1.y, w2 * c1.z);
    return vadd(vadd(p, a), b);
}

static cam_state cam_setup(const ro_camera *cam)
{
    cam_state cs;
    cs.c = ld3(cam->pos);
    cs.X = identity_rotate(ld3(cam->x_axis));
    cs.Y = identity_rotate(ld3(cam->y_axis));
    cs.Z = identity_rotate(ld3(cam->z_axis));
    /* camera.h:60: x_m(-w), x_inc((w * 2) / x_res) */
    cs.x_m = -cam->w;
    cs.y_m = -cam->h;
    cs.x_inc = (cam->w * 2.0f) / (float)cam->xres;
    cs.y_inc = (cam->h * 2.0f) / (float)cam->yres;
    cs.t = cam->t;
    return cs;
}

/* camera::pixel_to_co_ordinate (camera.h:127-140): no half-pixel offset. */
static inline ro_ray cam_ray(const cam_state *cs, int32_t x, int32_t y)
{
    const float x_t = ((float)x * cs->x_inc) + cs->x_m;
    const float y_t = ((float)y * cs->y_inc) + cs->y_m;
    const v3 screen = vadd(vadd(vmul(cs->X, x_t), vmul(cs->Y, y_t)), vmul(cs->Z, cs->t));
    ro_ray r = {cs->c, vnorm(screen)};
    return r;
}

void ro_camera_rays(const ro_camera *cam, int32_t x0, int32_t y0, int32_t w, int32_t h,
                    float *ogn, float *dir)
{
    const cam_state cs = cam_setup(cam);
    size_t k = 0;
    for (int32_t y = y0; y < y0 + h; ++y)
        for (int32_t x = x0; x < x0 + w; ++x, ++k) {
            const ro_ray r = cam_ray(&cs, x, y);
            ogn[3 * k] = r.o.x; ogn[3 * k + 1] = r.o.y; ogn[3 * k + 2] = r.o.z;
            dir[3 * k] = r.d.x; dir[3 * k + 1] = r.d.y; dir[3 * k + 2] = r.d.z;
        }
}

/* -------------------------------------------------------------- Shading */

/* ray::offset_start_point(+1) (ray.h:111-157): nudge each coordinate by
 * int(+-32 * n) units in the last place along the geometric normal, or by
 * 1e-4 * n (from zero) when the coordinate is tiny. */
static inline float offset_coord_d(float p, float n, float d)
{
    uint32_t x = f2u(p);
    if ((x & 0x7fffffffu) < f2u(RO_FP_DELTA_SMALL)) return 0.0f + (RO_FP_DELTA_SMALL * n);
    const float off = ((x >> 31) & 1u) ? -RO_FP_DELTA : RO_FP_DELTA;
    x += (uint32_t)cvtt((off * n) * d);
    return u2f(x);
}

static inline v3 offset_start(v3 dst, v3 geo)
{
    return mk(offset_coord_d(dst.x, geo.x, 1.0f), offset_coord_d(dst.y, geo.y, 1.0f),
              offset_coord_d(dst.z, geo.z, 1.0f));
}

/* offset_start_point(-1): into the surface (the refraction start point); the
 * tiny-coordinate case still steps along +n, as the reference does. */
static inline v3 offset_start_in(v3 dst, v3 geo)
{
    return mk(offset_coord_d(dst.x, geo.x, -1.0f), offset_coord_d(dst.y, geo.y, -1.0f),
              offset_coord_d(dst.z, geo.z, -1.0f));
}

/* A light light::find_rays treats as directional (light.h:65): not the
 * spherical / triangle constructors' n = (2, 2, 2), and no spot cone. */
static inline int light_is_directional(const ro_light *L)
{
    return L->kind == 1 || (L->kind == 2 && L->s_b == 0.0f);
}

/* Light direction sign for directional lights (light.h:172-219): the light
 * sits at +/-1e15 along n by the sign of n's major component. */
static float dir_light_dist(v3 n)
{
    if (fabsf(n.x) > fabsf(n.y)) {
        if (fabsf(n.x) > fabsf(n.z)) return (n.x < 0.0f) ? -1.0e15f : 1.0e15f;
        return (n.z < 0.0f) ? -1.0e15f : 1.0e15f;
    }
    if (fabsf(n.y) > fabsf(n.z)) return (n.y < 0.0f) ? -1.0e15f : 1.0e15f;
    return (n.z < 0.0f) ? -1.0e15f : 1.0e15f;
}

/* Shadow ray: ray::find_rays (ray.cc:91-104) -> light::find_rays
 * (light.h:62-100) -> ray::set_up(o, dst) (ray.h:44-54). */
static inline void shadow_ray(const ro_light *L, v3 start, ro_ray *r, float *len)
{
    v3 target;
    if (light_is_directional(L)) {
        const v3 n = ld3(L->dir);
        target = vadd(start, vmul(n, dir_light_dist(n)));
    } else {
        target = ld3(L->pos);
    }
    const v3 d = vsub(target, start);
    *len = vmag(d);
    r->o = start;
    r->d = vdivs(d, *len);
}

typedef struct {
    const ro_scene *s;
    const ro_camera *cam;
    const ro_light *lights;
    int32_t nlights;
    const ro_material *mat;       /* AO mode and material 0 */
    const ro_material *mats;      /* material table (ro_render_mt) */
    int32_t nmats;
    int32_t row0, row1;
    uint8_t *rgb;
    int32_t *hit_id;
    uint8_t *occl;
    float *fimg;
    int64_t rays;
    /* AO mode */
    int32_t ao_n;
    float ao_dist;
    uint32_t ao_seed;
    int32_t *ao_count;
    /* soft shadows (ro_render_soft): shadow rays per spherical light, the
     * frame's slice of the reference's random stream and, per pixel, the
     * index in it of the pixel's first number; per light the numbers a hit
     * draws and, for a triangle-defined light, the rays it makes */
    int32_t soft_n;
    const float *stream;
    const int64_t *px_draw;
    const int32_t *ldraw;
    const struct area_ray *const *area;
    int32_t next_row;
    pthread_mutex_t *lock;
} render_job;

/* ------------------------------------------------------ Soft shadows */

#define RO_PI 3.1415926535897932384626433f   /* common/common.cc:10 */
#define RO_COS_LUT_SIZE 16384                  /* COS_LUT_SIZE, common/common.h:109-111 */

/* static_cos (common/common.h:171-209): cos of size evenly spaced angles,
 * the angle rounded to binary32 and its cosine taken in double. */
static float g_cos_lut[RO_COS_LUT_SIZE];
static pthread_once_t g_cos_lut_once = PTHREAD_ONCE_INIT;
static void build_cos_lut(void)
{
    for (int32_t i = 0; i < RO_COS_LUT_SIZE; ++i)
        g_cos_lut[i] = (float)cos((double)((((float)i * 2.0f) * RO_PI) / (float)RO_COS_LUT_SIZE));
}

/* static_cos::get_cos / get_sin: the index truncates toward zero and wraps
 * modulo the table size (the unsigned conversion of a negative angle). */
static inline float lut_cos(float a)
{
    const float v = ((1.0f / (2.0f * RO_PI)) * (float)RO_COS_LUT_SIZE) * a;
    return g_cos_lut[(uint32_t)(int64_t)v & (RO_COS_LUT_SIZE - 1)];
}
static inline float lut_sin(float a) { return lut_cos(a - (RO_PI / 2.0f)); }

float ro_lut_cos(float a) { pthread_once(&g_cos_lut_once, build_cos_lut); return lut_cos(a); }
float ro_lut_sin(float a) { pthread_once(&g_cos_lut_once, build_cos_lut); return lut_sin(a); }

/* The reference's random generator (common/common.cc:35-105): a Mersenne
 * twister seeded with 5489 whose refill updates words 0..622 only, tempered
 * and scaled to [0, 1] in binary32. */
typedef struct { uint32_t mt[624]; int32_t idx; } ref_rng;

static void ref_rng_init(ref_rng *g)
{
    g->mt[0] = 5489u;
    for (int i = 1; i < 624; ++i) g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->idx = 624;
}

static void ref_rng_refill(ref_rng *g)
{
    uint32_t *mt = g->mt;
    for (int i = 0; i < 227; ++i) {
        const uint32_t y = (0x80000000u & mt[i]) + (0x7FFFFFFFu & mt[i + 1]);
        mt[i] = mt[i + 397] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    for (int i = 227; i < 623; ++i) {
        const uint32_t y = (0x80000000u & mt[i]) + (0x7FFFFFFFu & mt[i + 1]);
        mt[i] = mt[i - 227] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    g->idx = 0;
}

static inline float ref_rng_next(ref_rng *g)
{
    if (g->idx >= 624) ref_rng_refill(g);
    uint32_t y = g->mt[g->idx++];
    y ^= (y >> 11);
    y ^= ((y << 7) & 0x9d2c5680u);
    y ^= ((y << 15) & 0xefc60000u);
    y ^= (y >> 18);
    return (float)y * (1.0f / 4294967296.0f);
}

void ro_ref_random(int64_t start, int32_t n, float *out)
{
    ref_rng g;
    ref_rng_init(&g);
    for (int64_t i = 0; i < start; ++i) (void)ref_rng_next(&g);
    for (int32_t i = 0; i < n; ++i) out[i] = ref_rng_next(&g);
}

int32_t ro_area_light_rays(int32_t ntris, int32_t n, int32_t *cnt)
{
    if (ntris < 1 || n < 1) return -1;
    const int32_t ppt = n / ntris;
    const int32_t extra = n - ntris * ppt;
    const float stride = (float)ntris / (float)(extra > 1 ? extra : 1);
    float extra_point = 0.0f;
    int32_t made = 0;
    for (int32_t i = 0; i < ntris; ++i) {
        int32_t k = ppt;
        if (i == (int32_t)extra_point) {
            k = ppt + 1;
            extra_point += stride;
        }
        if (cnt) cnt[i] = k;
        made += k;
    }
    return made;
}

/* One ray a triangle-defined light makes: triangle tri's ray i of the cnt
 * it makes. */
typedef struct area_ray { int32_t tri, cnt, i; } area_ray;

/* Numbers one primary hit draws for light L with n soft-shadow rays: three
 * per ray of a spherical (point or spot) light, two per ray a triangle-
 * defined light makes (made), none for a directional light or n = 1. */
static inline int32_t soft_draws(const ro_light *L, int32_t n, int32_t made)
{
    if (n <= 1 || light_is_directional(L)) return 0;
    return L->ntris > 0 ? 2 * made : 3 * n;
}

/* A point of a triangle of a triangle-defined light (triangle::find_rays,
 * triangle.h:504-525): barycentrics beta, gamma from rnd[0..1], then
 * ray::set_up(start, point) (ray.h:44-54). */
static void area_light_ray(const ro_scene *s, const area_ray *e, v3 start, const float *rnd, ro_ray *r, float *len)
{
    const int32_t n = e->cnt, i = e->i;
    const float beta_scale = 1.0f / (float)((n >> 4) + ((n & 0xe) != 0) + 1);
    const float gamma_scale = 1.0f / (float)((n >> 4) + ((n & 0xc) != 0) + 1);
    const int32_t eighths = (i >> 2) & ~0x1;
    const float beta = rnd[0] * (beta_scale * (float)(eighths + (i & 0x1)));
    const float gamma = (rnd[1] * (gamma_scale * (float)(eighths + (i & 0x2)))) * (1.0f - beta);
    const float alpha = 1.0f - (beta + gamma);
    const v3 p = vadd(vadd(vmul(s->va[e->tri], alpha), vmul(s->vb[e->tri], beta)), vmul(s->vc[e->tri], gamma));
    const v3 d = vsub(p, start);
    *len = vmag(d);
    r->o = start;
    r->d = vdivs(d, *len);
}

/* Shadow ray i of n to spherical light L (light::find_rays, light.h:102-128):
 * a random offset of the light's centre drawn from rnd[0..2] (angles a and b,
 * radius), then ray::set_up(start, centre + offset) (ray.h:44-54). */
static void soft_ray(const ro_light *L, v3 start, int32_t n, int32_t i, const float *rnd, ro_ray *r, float *len)
{
    const float a_scale = 1.0f / (float)((n >> 4) + ((n & 0xe) != 0) + 1);
    const float b_scale = 1.0f / (float)((n >> 4) + ((n & 0xc) != 0) + 1);
    const float r_scale = 1.0f / (float)((n >> 4) + ((n & 0x8) != 0) + 1);
    const int32_t eighths = (i >> 2) & ~0x1;
    const float a_off = (rnd[0] * (a_scale * (float)(eighths + (i & 0x1)))) * (2.0f * RO_PI);
    const float b_off = (rnd[1] * (b_scale * (float)(eighths + (i & 0x2)))) * (2.0f * RO_PI);
    const float r_off = (rnd[2] * (r_scale * (float)(eighths + (i & 0x4)))) * L->r;
    const float sin_a = lut_sin(a_off), cos_a = lut_cos(a_off);
    const float sin_b = lut_sin(b_off), cos_b = lut_cos(b_off);
    const v3 off = mk((r_off * cos_a) * sin_b, (r_off * sin_a) * sin_b, r_off * cos_b);
    const v3 d = vsub(vadd(ld3(L->pos), off), start);
    *len = vmag(d);
    r->o = start;
    r->d = vdivs(d, *len);
}

/* Hit-point refinement + face-forwarding (raytracer.cc:30-31 and
 * triangle::normal_at_point, triangle.h:464-498), then the interpolated
 * attribute (triangle.h:74-79). */
static inline void hit_setup(const ro_scene *s, const ro_ray *r, int32_t id, const ro_hit *h,
                             v3 *dst, v3 *shader_n, v3 *geo, v3 *vt, int *out_in)
{
    v3 p = vadd(r->o, vmul(r->d, h->d));              /* calculate_destination */
    const v3 n = s->n[id];
    const float denom = vdot(n, r->d);
    const float num = vdot(n, vsub(s->vc[id], p));
    p = vadd(p, vmul(r->d, num / denom));              /* change_length */
    /* the shading normal interpolates the triangle's vertex normals when it
     * has them (triangle.h:473-476) */
    v3 sn = n;
    if (s->cn && s->cn[9 * (size_t)id] != RO_MAX_DIST) {
        const float *c = s->cn + 9 * (size_t)id;
        const float w = 1.0f - (h->u + h->v);
        sn = vadd(vadd(vmul(mk(c[6], c[7], c[8]), h->u), vmul(mk(c[3], c[4], c[5]), h->v)), vmul(mk(c[0], c[1], c[2]), w));
    }
    if (denom > 0.0f) { *shader_n = vneg(sn); *geo = vneg(n); }
    else { *shader_n = sn; *geo = n; }
    if (out_in) *out_in = !(denom > 0.0f);    /* hit_t::out_in: the ray enters the front face */
    *dst = p;
    if (s->ta) {
        const float w = 1.0f - (h->u + h->v);
        *vt = vadd(vadd(vmul(s->tc[id], h->u), vmul(s->tb[id], h->v)), vmul(s->ta[id], w));
    } else {
        *vt = mk(RO_MAX_DIST, RO_MAX_DIST, RO_MAX_DIST);
    }
}

/* Diffuse colour at the hit: coloured_mapper_shader.cc:61-66 with a texture
 * mapper that returns the attribute * 255. */
static inline v3 cur_kd(const ro_scene *s, const ro_material *m, v3 vt)
{
    v3 kd = ld3(m->kd);
    if (s->ta && !(m->flags & RO_MAT_NO_VERTEX_COLOUR)) {
        const v3 tex = mk(vt.x * 255.0f, vt.y * 255.0f, vt.z * 255.0f);
        const float k = 1.0f / 255.0f;
        kd = mk(tex.x * (m->kd[0] * k), tex.y * (m->kd[1] * k), tex.z * (m->kd[2] * k));
    }
    return kd;
}

/* camera::clip_image_to_rgb (camera.h:312-314): clamp then truncate. */
static inline uint8_t clip8(float v) { return (uint8_t)smin(255.0f, smax(0.0f, v / 1.0f)); }

/* MIN_REFLECTIVE_POWER (common/common.h:31), a double literal: the float
 * ray power is compared after promotion to double. */
#define RO_MIN_REFLECTIVE_POWER 0.1

/* One light's term of the coloured Phong (coloured_mapper_shader::shade,
 * coloured_mapper_shader.cc:76-112) added to c: ldir / len the light's
 * first shadow ray, lmagn the fraction of its rays that reached it, vd the
 * incoming ray's direction.  Nothing when the surface faces away. */
static void phong_term(const ro_light *L, v3 ldir, float len, float lmagn, v3 sn, v3 vd, v3 kd, v3 ks, float ns,
                       v3 *c)
{
    const float shade = vdot(ldir, sn);
    if (shade < 0.0f) return;
    const v3 ref = vsub(ldir, vmul(sn, 2.0f * shade));
    const float rdr = vdot(vd, ref);
    v3 sc = mk(shade * kd.x, shade * kd.y, shade * kd.z);
    if (rdr > 0.0f) {
        const float p = (float)pow((double)rdr, (double)ns);
        sc = mk(sc.x + p * ks.x, sc.y + p * ks.y, sc.z + p * ks.z);
    }
    /* light::get_light_intensity (light.h:44-59) */
    const float dist = len * L->d;
    const float d_scale = (dist * dist) + 1.0f;
    v3 I;
    if (L->kind == 2 && L->s_b != 0.0f) {
        /* spot light: falls off with the angle off its axis */
        const float a = acosf(vdot(ldir, ld3(L->dir)));
        const float p = (a - L->s_a) / (L->s_b - L->s_a);
        const float f = smax(0.0f, smin(1.0f, 1.0f - p));
        const float fs = f / d_scale;
        I = mk((L->rgb[0] / 255.0f) * fs, (L->rgb[1] / 255.0f) * fs, (L->rgb[2] / 255.0f) * fs);
    } else {
        I = mk((L->rgb[0] / 255.0f) / d_scale, (L->rgb[1] / 255.0f) / d_scale, (L->rgb[2] / 255.0f) / d_scale);
    }
    *c = mk(c->x + I.x * (sc.x * lmagn), c->y + I.y * (sc.y * lmagn), c->z + I.z * (sc.z * lmagn));
}

/* The colour of one ray (ray_trace_engine::ray_trace, raytracer.cc:20-87):
 * closest hit; hit refinement; one shadow ray per light; coloured Phong
 * (coloured_mapper_shader::shade, coloured_mapper_shader.cc:76-112); then,
 * for a reflective material, the mirror ray of ray::reflect (ray.cc:118-135:
 * power = magn * rf, traced while power > MIN_REFLECTIVE_POWER, direction
 * dir - n * (2 * dir.n), from the offset start point) whose colour, averaged
 * over its one ray, is added times rf (combind_secondary_rays,
 * coloured_mapper_shader.cc:117-122).  A miss is the background
 * (camera::shade, camera.h:236-239).  first: the camera ray (writes the
 * occlusion / AO outputs).  Returns the hit triangle or -1. */
static int32_t trace_colour(render_job *J, const ro_ray *r, float magn, int first, size_t pix, v3 *out)
{
    const ro_scene *s = J->s;
    ro_hit h;
    const int32_t id = closest(s, r, &h);
    J->rays += 1;
    if (!(h.d < RO_MAX_DIST)) {
        *out = ld3(J->cam->background);
        if (first && J->occl) J->occl[pix] = 0;
        if (first && J->ao_count) J->ao_count[pix] = 0;
        return id;
    }
    const ro_material *m = J->ao_n > 0 ? J->mat : &J->mats[s->mat ? s->mat[id] : 0];
    v3 dst, sn, geo, vt;
    int out_in;
    hit_setup(s, r, id, &h, &dst, &sn, &geo, &vt, &out_in);
    const v3 start = offset_start(dst, geo);
    const v3 kd = cur_kd(s, m, vt);
    const v3 ks = ld3(m->ks);
    v3 c = mk(0.0f, 0.0f, 0.0f);
    if (J->ao_n > 0) {
        /* AO mode: pixel = ka + kd * unoccluded fraction */
        float dirs[3 * 64], ogns[3 * 64];
        const float hp[3] = {dst.x, dst.y, dst.z}, gn[3] = {geo.x, geo.y, geo.z};
        ro_ao_rays(hp, gn, (uint32_t)pix, J->ao_n, J->ao_seed, ogns, dirs);
        int32_t made_it = 0;
        for (int32_t k = 0; k < J->ao_n; ++k) {
            ro_ray ar = {ld3(ogns + 3 * k), ld3(dirs + 3 * k)};
            if (!nearer(s, &ar, J->ao_dist)) ++made_it;
        }
        J->rays += J->ao_n;
        const float frac = (float)made_it / (float)J->ao_n;
        c = vadd(vmul(kd, frac), ld3(m->ka));
        if (J->ao_count) J->ao_count[pix] = made_it;
        *out = c;
        return id;
    }
    int64_t draw = (first && J->soft_n > 1) ? J->px_draw[pix] : 0;
    for (int32_t l = 0; l < J->nlights; ++l) {
        const ro_light *L = &J->lights[l];
        ro_ray sr;
        float len;
        int32_t nrays = 1, made = 0;
        if (first && J->ldraw && J->ldraw[l] > 0) {
            /* soft shadows: n rays to random points of the light, shaded with
             * the first one's direction and length (raytracer.cc:44-64) */
            nrays = J->soft_n;
            for (int32_t i = 0; i < nrays; ++i) {
                ro_ray ri;
                float li;
                if (J->area[l]) area_light_ray(s, &J->area[l][i], start, J->stream + draw + 2 * i, &ri, &li);
                else soft_ray(L, start, nrays, i, J->stream + draw + 3 * i, &ri, &li);
                if (i == 0) { sr = ri; len = li; }
                if (!nearer(s, &ri, li)) ++made;
            }
            draw += J->ldraw[l];
            J->rays += nrays;
        } else {
            shadow_ray(L, start, &sr, &len);
            const int occ = nearer(s, &sr, len);
            made = !occ;
            J->rays += 1;
            if (first && J->occl && l == 0) J->occl[pix] = (uint8_t)occ;
        }
        const float lmagn = (float)made / (float)nrays;   /* made_it / nr_pending_shadows */
        phong_term(L, sr.d, len, lmagn, sn, r->d, kd, ks, m->ns, &c);
    }
    c = vadd(c, ld3(m->ka));
    /* ray::reflect (ray.cc:118-135) */
    const float refl_power = magn * m->rf;
    int has_refl = 0;
    v3 refl_c = mk(0.0f, 0.0f, 0.0f);
    if ((double)refl_power > RO_MIN_REFLECTIVE_POWER) {
        const float rdn = 2.0f * vdot(r->d, sn);
        const ro_ray rr = {start, vsub(r->d, vmul(sn, rdn))};
        trace_colour(J, &rr, refl_power, 0, pix, &refl_c);
        has_refl = 1;
    }
    /* ray::refract (ray.cc:198-281): ri inverted for a ray entering the
     * front face, none beyond the critical angle, start point pushed into
     * the surface */
    const float refr_power = magn * m->tran;
    int has_refr = 0;
    v3 refr_c = mk(0.0f, 0.0f, 0.0f);
    if ((double)refr_power > RO_MIN_REFLECTIVE_POWER) {
        float ri = m->ri;
        const float rdn = -vdot(r->d, sn);
        if (out_in) ri = 1.0f / ri;
        const float cos_t2 = 1.0f - (ri * ri) * (1.0f - rdn * rdn);
        if (!(cos_t2 < 0.0f)) {
            const float off = ri * rdn - sqrtf(cos_t2);
            const ro_ray rr = {offset_start_in(dst, geo), vadd(vmul(r->d, ri), vmul(sn, off))};
            trace_colour(J, &rr, refr_power, 0, pix, &refr_c);
            has_refr = 1;
        }
    }
    /* combind_secondary_rays (coloured_mapper_shader.cc:117-130): the one
     * ray's average colour times rf, then times tran */
    if (m->rf > 0.0f && has_refl) c = vadd(c, vmul(vdivs(vadd(mk(0.0f, 0.0f, 0.0f), refl_c), 1.0f), m->rf));
    if (m->tran > 0.0f && has_refr) c = vadd(c, vmul(vdivs(vadd(mk(0.0f, 0.0f, 0.0f), refr_c), 1.0f), m->tran));
    *out = c;
    return id;
}

static void render_pixel(render_job *J, const cam_state *cs, int32_t x, int32_t y)
{
    const size_t pix = (size_t)x + (size_t)y * (size_t)J->cam->xres;
    const ro_ray r = cam_ray(cs, x, y);
    v3 c;
    const int32_t id = trace_colour(J, &r, 1.0f, 1, pix, &c);
    if (J->hit_id) J->hit_id[pix] = id;
    if (J->fimg) { J->fimg[3 * pix] = c.x; J->fimg[3 * pix + 1] = c.y; J->fimg[3 * pix + 2] = c.z; }
    J->rgb[3 * pix] = clip8(c.x);
    J->rgb[3 * pix + 1] = clip8(c.y);
    J->rgb[3 * pix + 2] = clip8(c.z);
}

static void *render_worker(void *arg)
{
    render_job *J0 = (render_job *)arg;
    render_job J = *J0;   /* private counters */
    J.rays = 0;
    const cam_state cs = cam_setup(J.cam);
    for (;;) {
        pthread_mutex_lock(J0->lock);
        const int32_t y = J0->next_row++;
        pthread_mutex_unlock(J0->lock);
        if (y >= J.row1) break;
        for (int32_t x = 0; x < J.cam->xres; ++x) render_pixel(&J, &cs, x, y);
    }
    pthread_mutex_lock(J0->lock);
    J0->rays += J.rays;
    pthread_mutex_unlock(J0->lock);
    return NULL;
}

static int64_t run_render(render_job *J, int32_t nthreads)
{
    pthread_mutex_t lock;
    pthread_mutex_init(&lock, NULL);
    J->lock = &lock;
    J->next_row = J->row0;
    J->rays = 0;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    int started = 0;
    for (int i = 1; i < nthreads; ++i)
        if (pthread_create(&th[started], NULL, render_worker, J) == 0) ++started;
    render_worker(J);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
    pthread_mutex_destroy(&lock);
    return J->rays;
}

int64_t ro_render(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                  const ro_material *mat, int32_t row0, int32_t row1, int32_t nthreads,
                  uint8_t *rgb, int32_t *hit_id, uint8_t *occl, float *fimg)
{
    if (!s || !s->nodes || !cam || !mat || !rgb || row0 < 0 || row1 > cam->yres || row0 > row1) return -1;
    render_job J;
    memset(&J, 0, sizeof(J));
    J.s = s; J.cam = cam; J.lights = lights; J.nlights = nlights; J.mat = mat; J.mats = mat; J.nmats = 1;
    J.row0 = row0; J.row1 = row1; J.rgb = rgb; J.hit_id = hit_id; J.occl = occl; J.fimg = fimg;
    return run_render(&J, nthreads);
}

int64_t ro_render_mt(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                     const ro_material *mats, int32_t nmats, int32_t row0, int32_t row1, int32_t nthreads,
                     uint8_t *rgb, int32_t *hit_id, uint8_t *occl, float *fimg)
{
    if (!s || !s->nodes || !cam || !mats || nmats < 1 || !rgb || row0 < 0 || row1 > cam->yres || row0 > row1)
        return -1;
    if (s->mat)
        for (int32_t i = 0; i < s->ntris; ++i)
            if (s->mat[i] < 0 || s->mat[i] >= nmats) return -1;
    render_job J;
    memset(&J, 0, sizeof(J));
    J.s = s; J.cam = cam; J.lights = lights; J.nlights = nlights; J.mat = mats; J.mats = mats; J.nmats = nmats;
    J.row0 = row0; J.row1 = row1; J.rgb = rgb; J.hit_id = hit_id; J.occl = occl; J.fimg = fimg;
    return run_render(&J, nthreads);
}

/* Pass 1 of a soft-shadow frame: 1 per pixel whose camera ray hits. */
typedef struct {
    const ro_scene *s;
    const ro_camera *cam;
    uint8_t *hit;
    int32_t next_row;
    pthread_mutex_t *lock;
} hit_job;

static void *hit_worker(void *arg)
{
    hit_job *H = (hit_job *)arg;
    const cam_state cs = cam_setup(H->cam);
    for (;;) {
        pthread_mutex_lock(H->lock);
        const int32_t y = H->next_row++;
        pthread_mutex_unlock(H->lock);
        if (y >= H->cam->yres) break;
        for (int32_t x = 0; x < H->cam->xres; ++x) {
            const ro_ray r = cam_ray(&cs, x, y);
            ro_hit h;
            (void)closest(H->s, &r, &h);
            H->hit[(size_t)x + (size_t)y * (size_t)H->cam->xres] = (uint8_t)(h.d < RO_MAX_DIST);
        }
    }
    return NULL;
}

int64_t ro_render_soft(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                       const ro_material *mats, int32_t nmats, int32_t samples, int64_t stream_offset,
                       int32_t nthreads, uint8_t *rgb, int32_t *hit_id, float *fimg, int64_t *stream_end)
{
    if (!s || !s->nodes || !cam || !mats || nmats < 1 || !rgb || samples < 1 || samples > 64 ||
        stream_offset < 0 || nlights < 0 || nlights > 64 || (nlights > 0 && !lights))
        return -1;
    /* per light: numbers a hit draws and, for a triangle-defined light, the
     * first `samples` rays it makes */
    int32_t ldraw[64];
    area_ray *area[64];
    memset(area, 0, sizeof(area));
    int bad = 0;
    for (int32_t l = 0; l < nlights && !bad; ++l) {
        const ro_light *L = &lights[l];
        int32_t made = 0;
        if (L->ntris > 0) {
            if (!L->tris || L->kind == 1 || L->r != 0.0f) { bad = 1; break; }
            for (int32_t j = 0; j < L->ntris; ++j)
                if (L->tris[j] < 0 || L->tris[j] >= s->ntris) bad = 1;
            if (bad) break;
            made = ro_area_light_rays(L->ntris, samples, NULL);
            if (samples > 1 && !light_is_directional(L)) {
                if (made < samples) { bad = 1; break; }
                int32_t *cnt = (int32_t *)malloc((size_t)L->ntris * sizeof(int32_t));
                area[l] = (area_ray *)malloc((size_t)made * sizeof(area_ray));
                if (!cnt || !area[l]) { free(cnt); bad = 1; break; }
                (void)ro_area_light_rays(L->ntris, samples, cnt);
                int32_t k = 0;
                for (int32_t j = 0; j < L->ntris; ++j)
                    for (int32_t i = 0; i < cnt[j]; ++i) {
                        area[l][k].tri = L->tris[j];
                        area[l][k].cnt = cnt[j];
                        area[l][k].i = i;
                        ++k;
                    }
                free(cnt);
            }
        } else if (L->ntris < 0) {
            bad = 1;
            break;
        }
        ldraw[l] = soft_draws(L, samples, made);
    }
    if (bad) {
        for (int32_t l = 0; l < nlights; ++l) free(area[l]);
        return -1;
    }
    for (int32_t i = 0; i < nmats; ++i)
        if (mats[i].rf > 0.0f || mats[i].tran > 0.0f) bad = 1;
    if (s->mat)
        for (int32_t i = 0; i < s->ntris; ++i)
            if (s->mat[i] < 0 || s->mat[i] >= nmats) bad = 1;
    pthread_once(&g_cos_lut_once, build_cos_lut);
    const size_t npix = (size_t)cam->xres * (size_t)cam->yres;
    uint8_t *hit = bad ? NULL : (uint8_t *)malloc(npix ? npix : 1);
    int64_t *px_draw = bad ? NULL : (int64_t *)malloc((npix ? npix : 1) * sizeof(int64_t));
    if (!hit || !px_draw) {
        free(hit);
        free(px_draw);
        for (int32_t l = 0; l < nlights; ++l) free(area[l]);
        return -1;
    }
    /* pass 1: which pixels hit */
    {
        pthread_mutex_t lock;
        pthread_mutex_init(&lock, NULL);
        hit_job H = {s, cam, hit, 0, &lock};
        if (nthreads < 1) nthreads = 1;
        if (nthreads > 256) nthreads = 256;
        pthread_t th[256];
        int started = 0;
        for (int i = 1; i < nthreads; ++i)
            if (pthread_create(&th[started], NULL, hit_worker, &H) == 0) ++started;
        hit_worker(&H);
        for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
        pthread_mutex_destroy(&lock);
    }
    /* each hit pixel draws the same count, in pixel order (x + y * xres:
     * ray_tracer's loops, y outer, raytracer.cc:586-592) */
    int32_t per_hit = 0;
    for (int32_t l = 0; l < nlights; ++l) per_hit += ldraw[l];
    int64_t total = 0;
    for (size_t p = 0; p < npix; ++p) {
        px_draw[p] = total;
        total += hit[p] ? per_hit : 0;
    }
    float *stream = (float *)malloc((size_t)(total > 0 ? total : 1) * sizeof(float));
    if (!stream) {
        free(hit);
        free(px_draw);
        for (int32_t l = 0; l < nlights; ++l) free(area[l]);
        return -1;
    }
    {
        ref_rng g;
        ref_rng_init(&g);
        for (int64_t i = 0; i < stream_offset; ++i) (void)ref_rng_next(&g);
        for (int64_t i = 0; i < total; ++i) stream[i] = ref_rng_next(&g);
    }
    render_job J;
    memset(&J, 0, sizeof(J));
    J.s = s; J.cam = cam; J.lights = lights; J.nlights = nlights; J.mat = mats; J.mats = mats; J.nmats = nmats;
    J.row0 = 0; J.row1 = cam->yres; J.rgb = rgb; J.hit_id = hit_id; J.fimg = fimg;
    J.soft_n = samples; J.stream = stream; J.px_draw = px_draw; J.ldraw = ldraw;
    J.area = (const area_ray *const *)area;
    const int64_t rays = run_render(&J, nthreads);
    for (int32_t l = 0; l < nlights; ++l) free(area[l]);
    free(stream);
    free(px_draw);
    free(hit);
    if (stream_end) *stream_end = stream_offset + total;
    return rays;
}

/* ------------------------------------------- Distributed ray tracing */

float ro_pixel_stream(uint64_t seed, uint32_t pixel, uint64_t node, uint32_t k)
{
    const uint32_t ctr[4] = {pixel, (uint32_t)node, (uint32_t)(node >> 32), k >> 2};
    uint32_t w[4];
    ro_philox4x32(ctr, (uint32_t)seed, (uint32_t)(seed >> 32), w);
    return (float)w[k & 3u] * (1.0f / 4294967296.0f);
}

/* SplitMix64's output function (Steele, Lea and Flood 2014; Vigna's
 * constants). */
static inline uint64_t splitmix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t ro_tree_child(uint64_t parent, int32_t set, int32_t index)
{
    return splitmix64(parent + (uint64_t)(set * 64 + index + 1) * 0x9E3779B97F4A7C15ull);
}

/* Where a node's numbers come from: the reference's generator (g), whose
 * order is the pixel's drawing order, or the pixel's stream of this tree
 * node. */
typedef struct {
    ref_rng *g;
    uint64_t seed;
    uint32_t pixel;
    uint64_t node;    /* RO_STREAM_PIXEL: the node drawing */
    uint32_t k;       /* numbers the node has drawn */
    int64_t *drawn;   /* numbers the pixel has drawn */
} draw_src;

static inline float draw_next(draw_src *S)
{
    const uint32_t k = S->k++;
    ++*S->drawn;
    return S->g ? ref_rng_next(S->g) : ro_pixel_stream(S->seed, S->pixel, S->node, k);
}

typedef struct {
    const ro_scene *s;
    const ro_camera *cam;
    const ro_light *lights;
    int32_t nlights;
    const ro_material *mats;
    int32_t nmats;
    ro_sampling smp;
    uint8_t *rgb;
    int32_t *hit_id;
    float *fimg;
    ref_rng *g;            /* RO_STREAM_REFERENCE */
    int64_t rays, drawn;
    int bad;               /* a case the reference cannot render (stale rays, componant overflow) */
    int32_t next_row;
    pthread_mutex_t *lock;
} dist_job;

/* A light's shadow rays at a hit (ray::find_rays, ray.cc:91-104 ->
 * light::find_rays, light.h:62-164): one to the centre for a directional
 * light or n = 1, else n rays to random points -- three numbers per ray of
 * a spherical light, two per ray a triangle-defined light makes (the first
 * n traced).  first / first_len: the first ray; returns the fraction that
 * reached the light. */
static float light_rays(dist_job *J, draw_src *S, const ro_light *L, v3 start, int32_t n, ro_ray *first,
                        float *first_len)
{
    const ro_scene *s = J->s;
    if (light_is_directional(L) || n == 1) {
        shadow_ray(L, start, first, first_len);
        J->rays += 1;
        return nearer(s, first, *first_len) ? 0.0f : 1.0f;
    }
    int32_t made = 0;
    if (L->ntris > 0) {
        const int32_t T = L->ntris, ppt = n / T, extra = n - T * ppt;
        const float stride = (float)T / (float)(extra > 1 ? extra : 1);
        float at = 0.0f;
        int32_t k = 0;
        for (int32_t j = 0; j < T; ++j) {
            int32_t cnt = ppt;
            if (j == (int32_t)at) {
                ++cnt;
                at += stride;
            }
            for (int32_t i = 0; i < cnt; ++i, ++k) {
                float rnd[2];
                rnd[0] = draw_next(S);
                rnd[1] = draw_next(S);
                if (k >= n) continue;   /* made, not traced */
                const area_ray e = {L->tris[j], cnt, i};
                ro_ray ri;
                float li;
                area_light_ray(s, &e, start, rnd, &ri, &li);
                if (k == 0) { *first = ri; *first_len = li; }
                if (!nearer(s, &ri, li)) ++made;
            }
        }
        if (k < n) J->bad = 1;   /* the reference would trace stale rays */
    } else {
        for (int32_t i = 0; i < n; ++i) {
            float rnd[3];
            rnd[0] = draw_next(S);
            rnd[1] = draw_next(S);
            rnd[2] = draw_next(S);
            ro_ray ri;
            float li;
            soft_ray(L, start, n, i, rnd, &ri, &li);
            if (i == 0) { *first = ri; *first_len = li; }
            if (!nearer(s, &ri, li)) ++made;
        }
    }
    J->rays += n;
    return (float)made / (float)n;
}

/* The rays of a reflection or refraction set about direction ref from
 * start (ray::reflect ray.cc:137-182, ray::refract ray.cc:236-280): one
 * ray along ref when the frame has no diffuse reflections or spread is 0;
 * else max(diffuse / comp, 1) rays ref + perpen * x + cross * y, with
 * perpen = (ref.z, ref.y, -ref.x), cross = ref x perpen, x, y = r cos a,
 * r sin a for r = spread * u1, a = 2 pi * u2 (through the cosine table);
 * directions are not normalised.  Returns the count; *child_comp the
 * rays' componant. */
static int32_t spread_rays(dist_job *J, draw_src *S, v3 start, v3 ref, float spread, int32_t comp, ro_ray *out,
                           int32_t *child_comp)
{
    if (J->smp.diffuse == 0 || spread == 0.0f) {
        out[0].o = start;
        out[0].d = ref;
        *child_comp = comp;
        return 1;
    }
    if (comp > (1 << 28)) {   /* comp << 2 would overflow the reference's int */
        J->bad = 1;
        *child_comp = comp;
        return 0;
    }
    *child_comp = comp << 2;
    const v3 perpen = mk(ref.z, ref.y, -ref.x);
    const v3 cross = mk((ref.y * perpen.z) - (ref.z * perpen.y), (ref.z * perpen.x) - (ref.x * perpen.z),
                        (ref.x * perpen.y) - (ref.y * perpen.x));
    int32_t nr = J->smp.diffuse / comp;
    if (nr < 1) nr = 1;
    for (int32_t i = 0; i < nr; ++i) {
        const float r_off = draw_next(S) * spread;
        const float a_off = draw_next(S) * (2.0f * RO_PI);
        const float x_off = r_off * lut_cos(a_off);
        const float y_off = r_off * lut_sin(a_off);
        out[i].o = start;
        out[i].d = vadd(vadd(ref, vmul(perpen, x_off)), vmul(cross, y_off));
    }
    return nr;
}

/* The colour of one ray of a distributed frame (see ro_render_distributed);
 * node: its tree node (RO_TREE_ROOT for the camera ray, ro_tree_child of
 * its parent's for the others). */
static int32_t dist_colour(dist_job *J, const draw_src *P, const ro_ray *r, float magn, int32_t comp, uint64_t node,
                           v3 *out)
{
    const ro_scene *s = J->s;
    draw_src N = *P;
    N.node = node;
    N.k = 0;
    draw_src *S = &N;
    ro_hit h;
    const int32_t id = closest(s, r, &h);
    J->rays += 1;
    if (!(h.d < RO_MAX_DIST)) {
        *out = ld3(J->cam->background);
        return id;
    }
    const ro_material *m = &J->mats[s->mat ? s->mat[id] : 0];
    v3 dst, sn, geo, vt;
    int out_in;
    hit_setup(s, r, id, &h, &dst, &sn, &geo, &vt, &out_in);
    const v3 start = offset_start(dst, geo);
    const v3 kd = cur_kd(s, m, vt);
    const v3 ks = ld3(m->ks);
    /* generate_rays: every light's rays, then the reflection and the
     * refraction sets (coloured_mapper_shader.cc:9-38) */
    int32_t n = J->smp.soft / comp;
    if (n < 1) n = 1;
    ro_ray lray[64];
    float llen[64], lmagn[64];
    for (int32_t l = 0; l < J->nlights; ++l) lmagn[l] = light_rays(J, S, &J->lights[l], start, n, &lray[l], &llen[l]);
    ro_ray refl[64], refr[64];
    int32_t nrefl = 0, nrefr = 0, comp_refl = comp, comp_refr = comp;
    const float refl_power = magn * m->rf;
    if ((double)refl_power > RO_MIN_REFLECTIVE_POWER) {
        const float rdn = 2.0f * vdot(r->d, sn);
        nrefl = spread_rays(J, S, start, vsub(r->d, vmul(sn, rdn)), m->rfd, comp, refl, &comp_refl);
    }
    const float refr_power = magn * m->tran;
    if ((double)refr_power > RO_MIN_REFLECTIVE_POWER) {
        float ri = m->ri;
        const float rdn = -vdot(r->d, sn);
        if (out_in) ri = 1.0f / ri;
        const float cos_t2 = 1.0f - (ri * ri) * (1.0f - rdn * rdn);
        if (!(cos_t2 < 0.0f)) {
            const float off = ri * rdn - sqrtf(cos_t2);
            nrefr = spread_rays(J, S, offset_start_in(dst, geo), vadd(vmul(r->d, ri), vmul(sn, off)), m->td, comp,
                                refr, &comp_refr);
        }
    }
    /* shade with each light's first ray and unoccluded fraction */
    v3 c = mk(0.0f, 0.0f, 0.0f);
    for (int32_t l = 0; l < J->nlights; ++l) phong_term(&J->lights[l], lray[l].d, llen[l], lmagn[l], sn, r->d, kd, ks,
                                                       m->ns, &c);
    c = vadd(c, ld3(m->ka));
    /* the secondary rays, in order, then their mean colours */
    v3 sum_refl = mk(0.0f, 0.0f, 0.0f), sum_refr = mk(0.0f, 0.0f, 0.0f);
    for (int32_t i = 0; i < nrefl && !J->bad; ++i) {
        v3 ci;
        (void)dist_colour(J, S, &refl[i], refl_power, comp_refl, ro_tree_child(node, 0, i), &ci);
        sum_refl = vadd(sum_refl, ci);
    }
    for (int32_t i = 0; i < nrefr && !J->bad; ++i) {
        v3 ci;
        (void)dist_colour(J, S, &refr[i], refr_power, comp_refr, ro_tree_child(node, 1, i), &ci);
        sum_refr = vadd(sum_refr, ci);
    }
    if (m->rf > 0.0f && nrefl > 0) c = vadd(c, vmul(vdivs(sum_refl, (float)nrefl), m->rf));
    if (m->tran > 0.0f && nrefr > 0) c = vadd(c, vmul(vdivs(sum_refr, (float)nrefr), m->tran));
    *out = c;
    return id;
}

static void dist_pixel(dist_job *J, const cam_state *cs, ref_rng *g, int32_t x, int32_t y)
{
    const size_t pix = (size_t)x + (size_t)y * (size_t)J->cam->xres;
    int64_t drawn = 0;
    const draw_src S = {g, J->smp.seed, (uint32_t)pix, RO_TREE_ROOT, 0u, &drawn};
    const ro_ray r = cam_ray(cs, x, y);
    v3 c;
    const int32_t id = dist_colour(J, &S, &r, 1.0f, 1, RO_TREE_ROOT, &c);
    J->drawn += drawn;
    if (J->hit_id) J->hit_id[pix] = id;
    if (J->fimg) { J->fimg[3 * pix] = c.x; J->fimg[3 * pix + 1] = c.y; J->fimg[3 * pix + 2] = c.z; }
    J->rgb[3 * pix] = clip8(c.x);
    J->rgb[3 * pix + 1] = clip8(c.y);
    J->rgb[3 * pix + 2] = clip8(c.z);
}

static void *dist_worker(void *arg)
{
    dist_job *J0 = (dist_job *)arg;
    dist_job J = *J0;   /* private counters */
    J.rays = 0;
    J.drawn = 0;
    J.bad = 0;
    const cam_state cs = cam_setup(J.cam);
    for (;;) {
        pthread_mutex_lock(J0->lock);
        const int32_t y = J0->next_row++;
        pthread_mutex_unlock(J0->lock);
        if (y >= J.cam->yres) break;
        for (int32_t x = 0; x < J.cam->xres; ++x) dist_pixel(&J, &cs, J.g, x, y);
    }
    pthread_mutex_lock(J0->lock);
    J0->rays += J.rays;
    J0->drawn += J.drawn;
    J0->bad |= J.bad;
    pthread_mutex_unlock(J0->lock);
    return NULL;
}

int64_t ro_render_distributed(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                              const ro_material *mats, int32_t nmats, const ro_sampling *smp, int32_t nthreads,
                              uint8_t *rgb, int32_t *hit_id, float *fimg, int64_t *drawn)
{
    if (!s || !s->nodes || !cam || !mats || nmats < 1 || !rgb || !smp || smp->soft < 1 || smp->soft > 64 ||
        smp->diffuse < 0 || smp->diffuse > 64 || nlights < 0 || nlights > 64 || (nlights > 0 && !lights) ||
        (smp->stream != RO_STREAM_REFERENCE && smp->stream != RO_STREAM_PIXEL) || smp->offset < 0)
        return -1;
    for (int32_t l = 0; l < nlights; ++l) {
        const ro_light *L = &lights[l];
        if (L->ntris < 0 || (L->ntris > 0 && (!L->tris || L->kind == 1 || L->r != 0.0f))) return -1;
        for (int32_t j = 0; j < L->ntris; ++j)
            if (L->tris[j] < 0 || L->tris[j] >= s->ntris) return -1;
    }
    for (int32_t i = 0; i < nmats; ++i)
        if (!(mats[i].rf >= 0.0f && mats[i].rf < 1.0f) || !(mats[i].tran >= 0.0f && mats[i].tran < 1.0f)) return -1;
    if (s->mat)
        for (int32_t i = 0; i < s->ntris; ++i)
            if (s->mat[i] < 0 || s->mat[i] >= nmats) return -1;
    pthread_once(&g_cos_lut_once, build_cos_lut);
    dist_job J;
    memset(&J, 0, sizeof(J));
    J.s = s; J.cam = cam; J.lights = lights; J.nlights = nlights; J.mats = mats; J.nmats = nmats; J.smp = *smp;
    J.rgb = rgb; J.hit_id = hit_id; J.fimg = fimg;
    ref_rng g;
    if (smp->stream == RO_STREAM_REFERENCE) {
        ref_rng_init(&g);
        for (int64_t i = 0; i < smp->offset; ++i) (void)ref_rng_next(&g);
        J.g = &g;
        nthreads = 1;   /* one stream drawn in pixel order */
    }
    pthread_mutex_t lock;
    pthread_mutex_init(&lock, NULL);
    J.lock = &lock;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    int started = 0;
    for (int i = 1; i < nthreads; ++i)
        if (pthread_create(&th[started], NULL, dist_worker, &J) == 0) ++started;
    dist_worker(&J);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
    pthread_mutex_destroy(&lock);
    if (J.bad) return -1;
    if (drawn) *drawn = J.drawn;
    return J.rays;
}

int32_t ro_scene_set_normals(ro_scene *s, const float *corner_normals)
{
    if (!s) return -1;
    free(s->cn);
    s->cn = NULL;
    if (!corner_normals) return 0;
    const size_t nt = (size_t)(s->ntris > 0 ? s->ntris : 1);
    s->cn = (float *)malloc(nt * 9 * sizeof(float));
    if (!s->cn) return -1;
    memcpy(s->cn, corner_normals, (size_t)s->ntris * 9 * sizeof(float));
    return 0;
}

int32_t ro_scene_set_materials(ro_scene *s, const int32_t *mat_of_tri)
{
    if (!s) return -1;
    free(s->mat);
    s->mat = NULL;
    if (!mat_of_tri) return 0;
    const size_t nt = (size_t)(s->ntris > 0 ? s->ntris : 1);
    s->mat = (int32_t *)malloc(nt * sizeof(int32_t));
    if (!s->mat) return -1;
    memcpy(s->mat, mat_of_tri, (size_t)s->ntris * sizeof(int32_t));
    return 0;
}

int64_t ro_render_ao(const ro_scene *s, const ro_camera *cam, const ro_material *mat,
                     int32_t nsamples, float ao_dist, uint32_t seed, int32_t row0, int32_t row1,
                     int32_t nthreads, uint8_t *rgb, int32_t *hit_id, int32_t *ao_count)
{
    if (!s || !s->nodes || !cam || !mat || !rgb || nsamples < 1 || nsamples > 64 || row0 < 0 ||
        row1 > cam->yres || row0 > row1)
        return -1;
    render_job J;
    memset(&J, 0, sizeof(J));
    J.s = s; J.cam = cam; J.mat = mat; J.row0 = row0; J.row1 = row1; J.rgb = rgb; J.hit_id = hit_id;
    J.ao_n = nsamples; J.ao_dist = ao_dist; J.ao_seed = seed; J.ao_count = ao_count;
    return run_render(&J, nthreads);
}

int32_t ro_pixel_secondary_rays(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                                int32_t ao_n, float ao_dist, uint32_t ao_seed, int32_t x, int32_t y,
                                int32_t *hit_id, float *ogn, float *dir, float *tmax)
{
    if (!s || !s->nodes || !cam || !hit_id || !ogn || !dir || !tmax || x < 0 || y < 0 || x >= cam->xres ||
        y >= cam->yres || ao_n < 0 || ao_n > 64 || nlights < 0 || nlights > 64 || (nlights > 0 && !lights))
        return -1;
    const cam_state cs = cam_setup(cam);
    const ro_ray r = cam_ray(&cs, x, y);
    ro_hit h;
    const int32_t id = closest(s, &r, &h);
    *hit_id = id;
    if (!(h.d < RO_MAX_DIST)) return 0;
    v3 dst, sn, geo, vt;
    int out_in;
    hit_setup(s, &r, id, &h, &dst, &sn, &geo, &vt, &out_in);
    if (ao_n > 0) {
        const float hp[3] = {dst.x, dst.y, dst.z}, gn[3] = {geo.x, geo.y, geo.z};
        const size_t pix = (size_t)x + (size_t)y * (size_t)cam->xres;
        ro_ao_rays(hp, gn, (uint32_t)pix, ao_n, ao_seed, ogn, dir);
        for (int32_t k = 0; k < ao_n; ++k) tmax[k] = ao_dist;
        return ao_n;
    }
    const v3 start = offset_start(dst, geo);
    for (int32_t l = 0; l < nlights; ++l) {
        ro_ray sr;
        float len;
        shadow_ray(&lights[l], start, &sr, &len);
        ogn[3 * l] = sr.o.x; ogn[3 * l + 1] = sr.o.y; ogn[3 * l + 2] = sr.o.z;
        dir[3 * l] = sr.d.x; dir[3 * l + 1] = sr.d.y; dir[3 * l + 2] = sr.d.z;
        tmax[l] = len;
    }
    return nlights;
}

/* ------------------------------------------------------- AO ray sampler */

/* Philox4x32-10 from Salmon, Moraes, Dror and Shaw, "Parallel random numbers:
 * as easy as 1, 2, 3" (SC'11): ten rounds of two 32x32->64 multiplies with a
 * Weyl-sequence key schedule. */
void ro_philox4x32(const uint32_t ctr[4], uint32_t key0, uint32_t key1, uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key0, k1 = key1;
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        const uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Cosine-weighted hemisphere directions about the geometric normal:
 * rejection-sampled unit disk (24-bit uniforms, at most 8 tries, else the
 * normal), lifted to the hemisphere (Malley's method), rotated by the
 * orthonormal basis of Duff et al., "Building an Orthonormal Basis,
 * Revisited" (JCGT 2017).  Only IEEE add/mul/div/sqrt, so every host and
 * the GPU produce the same bits.  Origin = offset_start_point(+1). */
void ro_ao_rays(const float hit_point[3], const float geo_normal[3], uint32_t pixel, int32_t nsamples,
                uint32_t seed, float *ogn, float *dir)
{
    const v3 g = ld3(geo_normal);
    const v3 start = offset_start(ld3(hit_point), g);
    const float sign = (g.z < 0.0f || (g.z == 0.0f && (f2u(g.z) >> 31))) ? -1.0f : 1.0f;
    const float a = -1.0f / (sign + g.z);
    const float b = (g.x * g.y) * a;
    const v3 T = mk(1.0f + ((sign * (g.x * g.x)) * a), sign * b, -(sign * g.x));
    const v3 B = mk(b, sign + ((g.y * g.y) * a), -g.y);
    for (int32_t s = 0; s < nsamples; ++s) {
        float x = 0.0f, y = 0.0f;
        int found = 0;
        for (uint32_t call = 0; call < 4 && !found; ++call) {
            const uint32_t ctr[4] = {pixel, (uint32_t)s, call, 0x414f5259u};
            uint32_t rnd[4];
            ro_philox4x32(ctr, seed, 0x52415054u, rnd);
            for (int pair = 0; pair < 2 && !found; ++pair) {
                const float px = ((float)(rnd[2 * pair] >> 8) * 1.1920928955078125e-7f) - 1.0f;
                const float py = ((float)(rnd[2 * pair + 1] >> 8) * 1.1920928955078125e-7f) - 1.0f;
                if (((px * px) + (py * py)) < 1.0f) { x = px; y = py; found = 1; }
            }
        }
        const float z = sqrtf(smax(0.0f, 1.0f - ((x * x) + (y * y))));
        const v3 d = vadd(vadd(vmul(T, x), vmul(B, y)), vmul(g, z));
        const v3 dn = vnorm(d);
        ogn[3 * s] = start.x; ogn[3 * s + 1] = start.y; ogn[3 * s + 2] = start.z;
        dir[3 * s] = dn.x; dir[3 * s + 1] = dn.y; dir[3 * s + 2] = dn.z;
    }
}

/* ------------------------------------------------------ Tone mapping */

/* RGB -> CIE XYZ rows and scotopic weights of camera::tone_map
 * (camera.cc:1127-1130). */
static const float TM_XB[3] = {0.4124f, 0.3576f, 0.1805f};
static const float TM_YB[3] = {0.2126f, 0.7151f, 0.0721f};
static const float TM_ZB[3] = {0.0193f, 0.1192f, 0.9505f};
static const float TM_VB[3] = {0.01477f, 0.497f, 0.631f};

/* camera::just_noticable_difference (camera.cc:1814-1840). */
static float tm_jnd(float La)
{
    const float lLa = log10f(La);
    float lLt;
    if (lLa < -3.94f) lLt = -2.86f;
    else if (lLa < -1.44f) lLt = powf((0.405f * lLa) + 1.6f, 2.18f) - 2.86f;
    else if (lLa < -0.0184f) lLt = lLa - 0.395f;
    else if (lLa < 1.9f) lLt = powf((0.249f * lLa) + 0.65f, 2.7f) - 0.72f;
    else lLt = lLa - 1.255f;
    return powf(10.0f, lLt);
}

#define RO_PI 3.1415926535897932384626433f

/* camera::histogram_tone_map (camera.cc:1843-2062) on the luminance (the g
 * channel, 3 floats per pixel) of a w*h frame: resample to one pixel per
 * degree of view, a 100-bin histogram of log luminance, trimmed against
 * a linear (or, human, the visibility-limited) ceiling until fewer than
 * 2.5 % of the pixels are trimmed, then every pixel mapped through the
 * cumulative histogram.  lw_avg: the log-average luminance (the contrast
 * fallback).  Returns silently for a black image, as the reference does. */
static void tm_histogram(float *img, int32_t w, int32_t h, const ro_tone_map *tm, int human, float lw_avg)
{
    const float x_m = -tm->cam_w, y_m = -tm->cam_h;
    const float x_angle = (-2.0f * x_m) / tm->cam_t;
    const float y_angle = (-2.0f * y_m) / tm->cam_t;
    const int sx = (int)(x_angle * (360.0f / (2.0f * RO_PI)));
    const int sy = (int)(y_angle * (360.0f / (2.0f * RO_PI)));
    float *sl = (float *)calloc((size_t)(sx > 0 ? sx : 1) * (size_t)(sy > 0 ? sy : 1), sizeof(float));
    if (!sl) return;
    const float inc_x = (float)w / (float)sx, inc_y = (float)h / (float)sy;
    float y0 = 0.0f, y1 = inc_y;
    for (int j = 0; j < sy; ++j) {
        float x0 = 0.0f, x1 = inc_x;
        for (int i = 0; i < sx; ++i) {
            float acc = 0.0f;
            for (int y = (int)y0; y <= (int)y1; ++y)
                for (int x = (int)x0; x <= (int)x1; ++x) acc += img[3 * ((size_t)y * w + x) + 1];
            sl[j * sx + i] = acc / (((x1 - x0) + 1.0f) * ((y1 - y0) + 1.0f));
            x0 = x1;
            x1 = smin((float)w - 1.0f, x1 + inc_x);
        }
        y0 = y1;
        y1 = smin((float)h - 1.0f, y1 + inc_y);
    }
    const int bins = 100;
    int pix_gt0 = 0;
    float lw_min = RO_MAX_DIST, lw_max = 0.0f;
    for (int i = 0; i < sx * sy; ++i)
        if (sl[i] > 0.0f) {
            lw_min = smin(lw_min, sl[i]);
            lw_max = smax(lw_max, sl[i]);
            ++pix_gt0;
        }
    if (lw_min <= 0.0f) { free(sl); return; }
    lw_min = smax(lw_min, 1.0e-4f);
    const float bw_min = logf(lw_min);
    float bw_max = logf(lw_max);
    if (bw_max == bw_min) bw_max += 0.0001f * fabsf(bw_max);
    const float ld_max = 300.0f, ld_min = 1.0f;
    const float bd_max = logf(ld_max), bd_min = logf(ld_min);
    const size_t n = (size_t)w * (size_t)h;
    if ((bd_max - bd_min) > (bw_max - bw_min)) {
        const float sf = (bd_max - bd_min) / (bw_max - bw_min);
        for (size_t i = 0; i < n; ++i) img[3 * i + 1] = (img[3 * i + 1] * sf) + bd_min;
        free(sl);
        return;
    }
    int his[101];
    float cdf[101];
    memset(his, 0, sizeof(his));
    memset(cdf, 0, sizeof(cdf));
    for (int i = 0; i < sx * sy; ++i)
        if (sl[i] > 0.0f) {
            int b = (int)(((logf(sl[i]) - bw_min) / (bw_max - bw_min)) * (float)bins) + 1;
            b = b < 0 ? 0 : (b > bins ? bins : b);
            his[b]++;
        }
    float sum = 0.0f;
    for (int i = 1; i <= bins; ++i) {
        sum += (float)his[i];
        cdf[i] = sum / (float)pix_gt0;
    }
    const float tolerance = 0.025f * (float)pix_gt0;
    const float bin_step = (bw_max - bw_min) / (float)bins;
    const float lw_step = (1.0f / (float)bins) * (bw_max - bw_min);
    int trimmings;
    for (int guard = 0; guard < 100000; ++guard) {
        trimmings = 0;
        if ((float)pix_gt0 < tolerance) {
            const float num = 1.219f + powf(ld_max * 0.5f, 0.4f);
            const float den = 1.219f + powf(lw_avg, 0.4f);
            const float sf = (1.0f / ld_max) * powf(num / den, 2.5f);
            for (size_t i = 0; i < n; ++i) img[3 * i + 1] *= sf;
            free(sl);
            return;
        }
        for (int i = 1; i <= bins; ++i) {
            float ceiling = ((float)pix_gt0 * bin_step) / (bd_max - bd_min);
            if (human) {
                const float bde = bd_min + ((bd_max - bd_min) * cdf[i]);
                const float ld = expf(bde);
                const float bw = ((float)i * lw_step) + bw_min;
                const float lw = expf(bw);
                ceiling *= (tm_jnd(ld) * lw) / (tm_jnd(lw) * ld);
            }
            if ((float)his[i] > ceiling) {
                trimmings += his[i] - (int)ceiling;
                his[i] = (int)ceiling;
            }
        }
        pix_gt0 = 0;
        for (int i = 1; i <= bins; ++i) pix_gt0 += his[i];
        sum = 0.0f;
        for (int i = 1; i <= bins; ++i) {
            sum += (float)his[i];
            cdf[i] = sum / (float)pix_gt0;
        }
        if (!((float)trimmings > tolerance)) break;
    }
    for (size_t i = 0; i < n; ++i) {
        const float g = img[3 * i + 1];
        if (g > 0.0f) {
            const float bw = logf(g);
            float bf = ((bw - bw_min) / (bw_max - bw_min)) * (float)bins;
            bf = smin(smax(bf, 0.0f), (float)bins);
            const int b0 = (int)bf;
            const int b1 = (b0 + 1) < bins ? (b0 + 1) : bins;
            const float s = bf - (float)b0;
            const float pbw = ((1.0f - s) * cdf[b0]) + (s * cdf[b1]);
            const float bde = bd_min + ((bd_max - bd_min) * pbw);
            img[3 * i + 1] = expf(bde) / ld_max;
        }
    }
    free(sl);
}

/* One discrete Fourier transform, sign -1 (forward) or +1, along axis ax of
 * a complex array (re, im) of dims n[0..2], row-major (the last fastest). */
static void dft_axis(double *re, double *im, const int32_t n[3], int ax, int sign)
{
    const int32_t m = n[ax];
    size_t inner = 1;
    for (int k = ax + 1; k < 3; ++k) inner *= (size_t)n[k];
    const size_t outer = ((size_t)n[0] * (size_t)n[1] * (size_t)n[2]) / ((size_t)m * inner);
    double *cs = (double *)malloc(2 * (size_t)m * sizeof(double));
    double *lr = (double *)malloc(4 * (size_t)m * sizeof(double));
    double *li = lr + m, *orr = lr + 2 * m, *oi = lr + 3 * m;
    for (int32_t k = 0; k < m; ++k) {
        const double a = 6.283185307179586476925286766559 * (double)k / (double)m;
        cs[2 * k] = cos(a);
        cs[2 * k + 1] = (double)sign * sin(a);
    }
    for (size_t o = 0; o < outer; ++o)
        for (size_t q = 0; q < inner; ++q) {
            const size_t base = o * (size_t)m * inner + q;
            for (int32_t j = 0; j < m; ++j) { lr[j] = re[base + (size_t)j * inner]; li[j] = im[base + (size_t)j * inner]; }
            for (int32_t k = 0; k < m; ++k) {
                double sr = 0.0, si = 0.0;
                for (int32_t j = 0; j < m; ++j) {
                    const int32_t t = (int32_t)(((int64_t)j * k) % m);
                    sr += lr[j] * cs[2 * t] - li[j] * cs[2 * t + 1];
                    si += lr[j] * cs[2 * t + 1] + li[j] * cs[2 * t];
                }
                orr[k] = sr;
                oi[k] = si;
            }
            for (int32_t k = 0; k < m; ++k) { re[base + (size_t)k * inner] = orr[k]; im[base + (size_t)k * inner] = oi[k]; }
        }
    free(lr);
    free(cs);
}

/* Circular convolution over dims n[0..2] (row-major) of nch real channels
 * (channel c at data + c * N) with kern, evaluated through the Fourier
 * transform in double: what the reference's single-precision FFTW plans
 * compute, without their rounding.  out: nch * N floats. */
static void circ_conv3(const float *data, int nch, const float *kern, const int32_t n[3], float *out)
{
    const size_t N = (size_t)n[0] * (size_t)n[1] * (size_t)n[2];
    double *kr = (double *)calloc(2 * N, sizeof(double)), *ki = kr + N;
    double *dr = (double *)calloc(2 * N, sizeof(double)), *di = dr + N;
    for (size_t i = 0; i < N; ++i) kr[i] = kern[i];
    for (int ax = 0; ax < 3; ++ax) dft_axis(kr, ki, n, ax, -1);
    for (int c = 0; c < nch; ++c) {
        for (size_t i = 0; i < N; ++i) { dr[i] = data[(size_t)c * N + i]; di[i] = 0.0; }
        for (int ax = 0; ax < 3; ++ax) dft_axis(dr, di, n, ax, -1);
        for (size_t i = 0; i < N; ++i) {
            const double a = dr[i] * kr[i] - di[i] * ki[i], b = dr[i] * ki[i] + di[i] * kr[i];
            dr[i] = a;
            di[i] = b;
        }
        for (int ax = 0; ax < 3; ++ax) dft_axis(dr, di, n, ax, +1);
        for (size_t i = 0; i < N; ++i) out[(size_t)c * N + i] = (float)(dr[i] / (double)N);
    }
    free(dr);
    free(kr);
}

/* camera::bilateral_filter_tone_map(0.4, s, 0.4, s), s = 0.02 * min(w, h)
 * (camera.cc:1354-1358, 1632-1812): the bilateral grid of log10 luminance
 * (one cell per s pixels and per 0.4 decades, 3 cells of padding), blurred
 * by a Gaussian of one cell through a Fourier-domain product, sliced
 * trilinearly at every pixel, then the detail (log luminance less the
 * blurred base) kept and the base compressed to a contrast of 300:
 * Y = 10^(base * gamma + detail) / 255.  The reference hands its
 * x-fastest grid (index x + W (y + H z)) to FFTW as dims (W, H, D), whose
 * last dimension varies fastest, so its "Gaussian" is convolved over those
 * axes of the flat array; restated as such.  A pixel at or below 3.18e-7
 * has no log value in the reference (its array is left unset there): here
 * it is 0, what a glibc host's fresh pages hold for frames over 32,768
 * pixels, and its grid cell is clamped into the grid. */
static void tm_bilateral(float *img, int32_t w, int32_t h)
{
    const int32_t n = w * h;
    const float r_s = 0.4f, s_s = 0.02f * (float)(w < h ? w : h), r_sa = 0.4f, s_sa = s_s;
    float *logi = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
    float in_max = -RO_MAX_DIST, in_min = RO_MAX_DIST;
    for (int32_t i = 0; i < n; ++i) {
        const float g = img[3 * (size_t)i + 1];
        if (g > 3.18e-7f) {
            logi[i] = log10f(g);
            in_max = smax(in_max, logi[i]);
            in_min = smin(in_min, logi[i]);
        } else {
            logi[i] = 0.0f;
        }
    }
    const float delta = in_max - in_min;
    const float sigma_r = r_s / r_sa, sigma_s = s_s / s_sa;
    const int32_t pxy = (int32_t)(2.0f * sigma_s) + 1, pz = (int32_t)(2.0f * sigma_r) + 1;
    const int32_t W = (int32_t)((float)(w - 1) / s_sa) + 1 + (pxy << 1);
    const int32_t H = (int32_t)((float)(h - 1) / s_sa) + 1 + (pxy << 1);
    const int32_t D = (int32_t)(delta / r_sa) + 1 + (pz << 1);
    const size_t N = (size_t)W * (size_t)H * (size_t)D;
    float *wiw = (float *)calloc(2 * N, sizeof(float));
    for (int32_t x = 0; x < w; ++x)
        for (int32_t y = 0; y < h; ++y) {
            const int32_t sx = (int32_t)((float)x / s_sa + 0.5f) + pxy;
            const int32_t sy = (int32_t)((float)y / s_sa + 0.5f) + pxy;
            int32_t sz = (int32_t)((logi[x + w * y] - in_min) / r_sa + 0.5f) + pz;
            sz = sz < 0 ? 0 : (sz > D - 1 ? D - 1 : sz);
            const size_t c = (size_t)sx + (size_t)W * ((size_t)sy + (size_t)H * (size_t)sz);
            wiw[c] += 1.0f;
            wiw[c + N] += logi[x + w * y];
        }
    float *kern = (float *)malloc(N * sizeof(float));
    const int32_t hw = W >> 1, hh = H >> 1, hd = D >> 1;
    for (int32_t x = 0; x < W; ++x) {
        const float X = (float)x - ((x > hw) ? (float)W : 0.0f);
        for (int32_t y = 0; y < H; ++y) {
            const float Y = (float)y - ((y > hh) ? (float)H : 0.0f);
            for (int32_t z = 0; z < D; ++z) {
                const float Z = (float)z - ((z > hd) ? (float)D : 0.0f);
                const float rr = ((X * X) + (Y * Y)) / (sigma_s * sigma_s) + (Z * Z) / (sigma_r * sigma_r);
                kern[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * (size_t)z)] = expf(-rr * 0.5f);
            }
        }
    }
    float *blur = (float *)malloc(2 * N * sizeof(float));
    const int32_t dims[3] = {W, H, D};
    circ_conv3(wiw, 2, kern, dims, blur);
    const float *bw = blur, *biw = blur + N;
    float *res = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
    float max_v = -RO_MAX_DIST, min_v = RO_MAX_DIST;
    for (int32_t x = 0; x < w; ++x)
        for (int32_t y = 0; y < h; ++y) {
            const float z = logi[x + w * y] - in_min;
            const float xa_ = (float)x / s_sa + (float)pxy;
            const int32_t xi = (int32_t)xa_ < W - 1 ? (int32_t)xa_ : W - 1, xi0 = xi < 0 ? 0 : xi;
            const int32_t xx = xi0 + 1 < W - 1 ? xi0 + 1 : W - 1;
            const float ya_ = (float)y / s_sa + (float)pxy;
            const int32_t yi = (int32_t)ya_ < H - 1 ? (int32_t)ya_ : H - 1, yi0 = yi < 0 ? 0 : yi;
            const int32_t yy = yi0 + 1 < H - 1 ? yi0 + 1 : H - 1;
            const float za_ = z / r_sa + (float)pz;
            const int32_t zi = (int32_t)za_ < D - 1 ? (int32_t)za_ : D - 1, zi0 = zi < 0 ? 0 : zi;
            const int32_t zz = zi0 + 1 < D - 1 ? zi0 + 1 : D - 1;
            const float ax = xa_ - (float)xi0, ay = ya_ - (float)yi0, az = za_ - (float)zi0;
#define RO_AT(A, X_, Y_, Z_) (A)[(size_t)(X_) + (size_t)W * ((size_t)(Y_) + (size_t)H * (size_t)(Z_))]
            const float IW = (1.0f - ax) * (1.0f - ay) * (1.0f - az) * RO_AT(biw, xi0, yi0, zi0) +
                             ax * (1.0f - ay) * (1.0f - az) * RO_AT(biw, xx, yi0, zi0) +
                             (1.0f - ax) * ay * (1.0f - az) * RO_AT(biw, xi0, yy, zi0) +
                             ax * ay * (1.0f - az) * RO_AT(biw, xx, yy, zi0) +
                             (1.0f - ax) * (1.0f - ay) * az * RO_AT(biw, xi0, yi0, zz) +
                             ax * (1.0f - ay) * az * RO_AT(biw, xx, yi0, zz) +
                             (1.0f - ax) * ay * az * RO_AT(biw, xi0, yy, zz) +
                             ax * ay * az * RO_AT(biw, xx, yy, zz);
            const float Wt = (1.0f - ax) * (1.0f - ay) * (1.0f - az) * RO_AT(bw, xi0, yi0, zi0) +
                             ax * (1.0f - ay) * (1.0f - az) * RO_AT(bw, xx, yi0, zi0) +
                             (1.0f - ax) * ay * (1.0f - az) * RO_AT(bw, xi0, yy, zi0) +
                             ax * ay * (1.0f - az) * RO_AT(bw, xx, yy, zi0) +
                             (1.0f - ax) * (1.0f - ay) * az * RO_AT(bw, xi0, yi0, zz) +
                             ax * (1.0f - ay) * az * RO_AT(bw, xx, yi0, zz) +
                             (1.0f - ax) * ay * az * RO_AT(bw, xi0, yy, zz) +
                             ax * ay * az * RO_AT(bw, xx, yy, zz);
#undef RO_AT
            const float r = IW / Wt;
            res[x + w * y] = r;
            max_v = smax(max_v, r);
            min_v = smin(min_v, r);
        }
    const float contrast = 300.0f;
    const float gamma = log10f(contrast) / (max_v - min_v);
    for (int32_t i = 0; i < n; ++i) {
        const float scaled = powf(10.0f, (res[i] * gamma + (logi[i] - res[i])));
        img[3 * (size_t)i + 1] = scaled * (1.0f / 255.0f);
    }
    free(res);
    free(blur);
    free(kern);
    free(wiw);
    free(logi);
}

int32_t ro_tone_map_frame(float *img, int32_t w, int32_t h, const ro_tone_map *tm)
{
    const int32_t mode = tm->mode;
    if (!(mode >= 0 && mode <= 9)) return -1;
    const int32_t n = w * h;
    /* first pass: to CIE Yxy, log-average and maximum luminance */
    float Yi = 0.0f, maxY = 0.0f, rgbAvg = 0.0f;
    int numpix = 0;
    for (int32_t i = 0; i < n; ++i) {
        float *p = img + 3 * (size_t)i;
        const float r = p[0] / 255.0f, g = p[1] / 255.0f, b = p[2] / 255.0f;
        if (mode == 5) rgbAvg += (r + g + b) * (1.0f / 3.0f);
        const float X = 683.0f * (((TM_XB[0] * r) + (TM_XB[1] * g)) + (TM_XB[2] * b));
        float Y = 683.0f * (((TM_YB[0] * r) + (TM_YB[1] * g)) + (TM_YB[2] * b));
        const float Z = 683.0f * (((TM_ZB[0] * r) + (TM_ZB[1] * g)) + (TM_ZB[2] * b));
        if (Y < 3.18e-7f) {
            Y = 3.18e-7f;
        } else {
            numpix++;
            maxY = smax(maxY, Y);
            Yi += log10f(Y);
        }
        const float W = (Y + X) + Z;
        float x = X / W, y = Y / W;
        if (tm->desaturate) {
            float s;
            const float l = log10f(Y);
            if (l < -2.0f) {
                s = 0.0f;
            } else if (l < 0.6f) {
                const float q = (l + 2.0f) / 2.6f;
                const float q2 = q * q;
                s = (3.0f * q2) - ((2.0f * q) * q2);
            } else {
                s = 1.0f;
            }
            const float V = 1700.0f * (((TM_VB[0] * r) + (TM_VB[1] * g)) + (TM_VB[2] * b));
            x = ((1.0f - s) * tm->xw) + (s * ((x + tm->xw) - (1.0f / 3.0f)));
            y = ((1.0f - s) * tm->yw) + (s * ((y + tm->yw) - (1.0f / 3.0f)));
            Y = ((0.4468f * (1.0f - s)) * V) + (s * Y);
        }
        p[0] = x;
        p[1] = Y;
        p[2] = y;
    }
    if (numpix) Yi /= (float)numpix;
    rgbAvg /= (float)(uint32_t)n;
    Yi = powf(10.0f, Yi);
    /* luminance scaling by mode (camera.cc:1276-1425) */
    const float key = tm->key;
    if (mode == 1) {
        const float Yw = 300.0f;
        const float num = 1.219f + powf(Yw * 0.5f, 0.4f);
        const float den = 1.219f + powf(Yi, 0.4f);
        const float sf = (1.0f / Yw) * powf(num / den, 2.5f);
        for (int32_t i = 0; i < n; ++i) img[3 * (size_t)i + 1] *= sf;
    } else if (mode == 4) {
        const float sf = key / Yi;
        maxY *= sf;
        maxY = 1.0f / (maxY * maxY);
        for (int32_t i = 0; i < n; ++i) {
            float g = img[3 * (size_t)i + 1] * sf;
            if (maxY != 0.0f) g *= (1.0f + (g * maxY)) / (1.0f + g);
            img[3 * (size_t)i + 1] = g;
        }
    } else if (mode == 5) {
        const float sf = key / Yi;
        maxY *= sf;
        for (int32_t i = 0; i < n; ++i) {
            float g = img[3 * (size_t)i + 1] * sf;
            if (maxY != 0.0f) g = 1.0f - expf(-g);
            img[3 * (size_t)i + 1] = g;
        }
    } else if (mode == 6) {
        /* rgbAvg is only accumulated in exposure mode (camera.cc:1142), so
         * here it is 0 and the scale stays 1, as in the reference */
        float sf = 1.0f;
        if (rgbAvg != 0.0f) sf *= key * (0.5f / (rgbAvg * 683.0f));
        for (int32_t i = 0; i < n; ++i) img[3 * (size_t)i + 1] *= sf;
    } else if (mode == 7) {
        const float sf = key / maxY;
        for (int32_t i = 0; i < n; ++i) img[3 * (size_t)i + 1] *= sf;
    } else if (mode == 2 || mode == 3) {
        tm_histogram(img, w, h, tm, mode == 3, Yi);
    } else if (mode == 8) {
        tm_bilateral(img, w, h);
    } else if (mode == 9) {
        const float lda = 800.0f;
        const float log_lda = logf(lda * 0.5f);
        const float log_la = logf(Yi);
        float tp, ts, k;
        if (log_la <= -2.6f) tp = -0.72f;
        else if (log_la <= 1.9f) tp = powf((0.249f * log_la) + 0.65f, 2.7f) - 0.72f;
        else tp = log_la - 1.255f;
        const float mp = (log_lda - 1.255f) / tp;
        if (log_la <= -3.94f) ts = -2.86f;
        else if (log_la < -1.44f) ts = powf((0.405f * log_la) + 1.6f, 2.18f) - 2.86f;
        else ts = log_la - 0.395f;
        const float ms = (log_lda - 1.255f) / ts;
        if (log_la < -2.0f) k = 1.0f;
        else if (log_la < 1.0f) k = 1.0f - ((log_la + 2.0f) * (1.0f / 3.0f));
        else k = 0.0f;
        for (int32_t i = 0; i < n; ++i) {
            const float g = img[3 * (size_t)i + 1];
            const float ldp = mp * g, lds = ms * g;
            img[3 * (size_t)i + 1] = (1.0f / lda) * (ldp + (k * lds));
        }
    } else {
        const float sf = 1.0f / 683.0f;
        for (int32_t i = 0; i < n; ++i) img[3 * (size_t)i + 1] *= sf;
    }
    /* contrast stretch (camera.cc:1428-1450) */
    if (tm->stretch) {
        float maxY2 = -RO_MAX_DIST, minY2 = RO_MAX_DIST;
        for (int32_t i = 0; i < n; ++i) {
            maxY2 = smax(maxY2, img[3 * (size_t)i + 1]);
            minY2 = smin(minY2, img[3 * (size_t)i + 1]);
        }
        if (((minY2 > 0.0f) || (maxY2 < 0.0f)) && (minY2 < maxY2)) {
            const float offset = smin(-minY2, 0.0f);
            const float scale = 1.0f / (smin(1.0f, maxY2) - smax(0.0f, minY2));
            for (int32_t i = 0; i < n; ++i) img[3 * (size_t)i + 1] = (img[3 * (size_t)i + 1] + offset) * scale;
        }
    }
    /* Yxy -> RGB in 0..255 (camera.cc:2080-2098), then gamma (camera.cc:1466-1500) */
    for (int32_t i = 0; i < n; ++i) {
        float *p = img + 3 * (size_t)i;
        const float x = p[0], Y = p[1], y = p[2];
        const float X = (x * Y) / y;
        const float Z = (((1.0f - x) - y) * Y) / y;
        float r = ((826.353f * X) + (-391.986f * Y)) + (-127.143f * Z);
        float g = ((-247.0695f * X) + (478.329f * Y)) + (10.5825f * Z);
        float b = ((14.2035f * X) + (-52.02f * Y)) + (269.535f * Z);
        if (tm->gamma > 0.0f) {
            const float gm = tm->gamma;
            float c[3] = {r / 255.0f, g / 255.0f, b / 255.0f};
            for (int k = 0; k < 3; ++k) {
                c[k] = smin(smax(c[k], 0.0f), 1.0f);
                if (fabsf(gm - 2.2f) > 0.001f) c[k] = powf(c[k], 1.0f / gm);
                else if (fabsf(gm - 1.0f) > 0.001f)
                    c[k] = (c[k] <= 0.0031308f) ? (12.92f * c[k]) : ((1.055f * powf(c[k], 1.0f / 2.4f)) - 0.055f);
            }
            r = c[0] * 255.0f;
            g = c[1] * 255.0f;
            b = c[2] * 255.0f;
        }
        p[0] = r;
        p[1] = g;
        p[2] = b;
    }
    return 0;
}
