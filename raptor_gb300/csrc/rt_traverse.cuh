// rt_traverse.cuh -- per-ray traversal of the 8-wide quantised BVH, the
// reference-exact Moller-Trumbore test, and the shading helpers shared by
// every kernel of the core.
//
// Traversal keeps node groups (child base + hit bits) on a per-ray stack:
// internal-child hits live in bits 24..31 at position (slot ^ octant) so the
// lowest set bit is the child nearest the ray's origin side, the node's
// internal-child mask rides in bits 0..7, and leaf triangles of a node are
// tested as soon as the node is intersected (after Ylitie et al., HPG 2017).
#pragma once

#include "rt_internal.cuh"

namespace rtc {

struct RayState {
    float3 o, d;
};

// Reference-exact triangle test (triangle::is_intersecting,
// raytracer/triangle.h:190-235): e1 = c - a, e2 = b - a, reject
// |det| < 1e-6, u weighs c, v weighs b.  Returns t, or +inf when rejected.
__device__ __forceinline__ float mt_intersect(const float4 w0, const float4 w1, const float4 w2, const float3 o,
                                              const float3 d, float &u_out, float &v_out)
{
    const float3 a = make_float3(w0.x, w0.y, w0.z);
    const float3 b = make_float3(w0.w, w1.x, w1.y);
    const float3 c = make_float3(w1.z, w1.w, w2.x);
    const float3 e1 = xsub3(c, a);   // triangle.h:193
    const float3 e2 = xsub3(b, a);   // triangle.h:194
    const float3 P = xcross(d, e2);
    const float det = xdot(e1, P);
    const float inv_det = __frcp_rn(det);      // == 1.0f / det, correctly rounded
    const float3 T = xsub3(o, a);
    const float u = xmul(xdot(T, P), inv_det);
    const float3 Q = xcross(T, e1);
    const float v = xmul(xdot(d, Q), inv_det);
    const float t = xmul(xdot(e2, Q), inv_det);
    const bool reject = (det > -kDetEps && det < kDetEps) || (u < 0.0f) || (v < 0.0f) || (xadd(u, v) > 1.0f);
    u_out = u;
    v_out = v;
    return reject ? __int_as_float(0x7f800000) : t;
}

// Per-ray constants of the watertight test: the axis of largest |d| is z
// (kx, ky follow, swapped when d.z < 0 to keep the winding), and the shear
// that maps the ray to +z.
struct Shear {
    int kx, ky, kz;
    float sx, sy, sz;
};

__device__ __forceinline__ float comp(const float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ Shear make_shear(const float3 d)
{
    Shear s;
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    s.kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    s.kx = (s.kz + 1) % 3;
    s.ky = (s.kx + 1) % 3;
    if (comp(d, s.kz) < 0.0f) { const int t = s.kx; s.kx = s.ky; s.ky = t; }
    const float dz = comp(d, s.kz);
    s.sx = comp(d, s.kx) / dz;
    s.sy = comp(d, s.ky) / dz;
    s.sz = 1.0f / dz;
    return s;
}

// Watertight ray/triangle test of Woop, Benthin and Wald (JCGT 2013): the
// three edge functions are evaluated in the ray's sheared frame from the
// exact vertex positions, so two triangles sharing an edge always agree on
// which side a ray passes (no ray leaks through a shared edge); an edge
// function that rounds to exactly zero is re-evaluated in double.  Returns
// t (accepting t > 0 here; the caller applies EPSILON), or +inf.  u weighs
// c and v weighs b, as in the reference.
__device__ __forceinline__ float wt_intersect(const float4 w0, const float4 w1, const float4 w2, const float3 o,
                                              const Shear &sh, float &u_out, float &v_out)
{
    const float3 A = make_float3(w0.x - o.x, w0.y - o.y, w0.z - o.z);
    const float3 B = make_float3(w0.w - o.x, w1.x - o.y, w1.y - o.z);
    const float3 C = make_float3(w1.z - o.x, w1.w - o.y, w2.x - o.z);
    const float Az = comp(A, sh.kz), Bz = comp(B, sh.kz), Cz = comp(C, sh.kz);
    // every vertex is sheared by the same uncontracted operations, so a
    // vertex shared by several triangles lands on the same point in all
    const float Ax = xsub(comp(A, sh.kx), xmul(sh.sx, Az)), Ay = xsub(comp(A, sh.ky), xmul(sh.sy, Az));
    const float Bx = xsub(comp(B, sh.kx), xmul(sh.sx, Bz)), By = xsub(comp(B, sh.ky), xmul(sh.sy, Bz));
    const float Cx = xsub(comp(C, sh.kx), xmul(sh.sx, Cz)), Cy = xsub(comp(C, sh.ky), xmul(sh.sy, Cz));
    // uncontracted products: an edge shared by two triangles gives exactly
    // negated edge functions in both
    float U = xsub(xmul(Cx, By), xmul(Cy, Bx));
    float V = xsub(xmul(Ax, Cy), xmul(Ay, Cx));
    float W = xsub(xmul(Bx, Ay), xmul(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    const float inf = __int_as_float(0x7f800000);
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return inf;
    const float det = U + V + W;
    if (det == 0.0f) return inf;
    const float T = (U * (sh.sz * Az) + V * (sh.sz * Bz)) + W * (sh.sz * Cz);
    const float inv = 1.0f / det;
    const float t = T * inv;
    if (!(t > 0.0f)) return inf;
    u_out = W * inv;   // weight of c
    v_out = V * inv;   // weight of b
    return t;
}

// Out-of-line entry to the watertight test (shear set up per call), so the
// default reference-exact path keeps its registers.
static __device__ __noinline__ float wt_intersect_ray(const float4 w0, const float4 w1, const float4 w2, const float3 o,
                                               const float3 d, float *u_out, float *v_out)
{
    const Shear sh = make_shear(d);
    float u = 0.f, v = 0.f;
    const float t = wt_intersect(w0, w1, w2, o, sh, u, v);
    *u_out = u;
    *v_out = v;
    return t;
}

// Child-box test of one wide node: returns internal-hit bits (24..31,
// permuted by octant) | imask (0..7) in .y with child_base in .x, and the
// triangle-hit bits (0..23) with tri_base in tgroup.
struct NodeHits {
    uint2 ngroup;
    uint2 tgroup;
};

__device__ __forceinline__ uint32_t byte_of(uint32_t lo, uint32_t hi, int s)
{
    return ((s < 4) ? (lo >> (8 * s)) : (hi >> (8 * (s - 4)))) & 0xffu;
}

// Quantised byte s of a 64-bit plane as a float.  RT_NODE_PRMT: one byte
// permute places q in mantissa bits 8..15 of 1.0f, giving exactly
// 1 + q * 2^-15; intersect_node folds the constant 1 into the node's offset
// (kQOne below), so a plane costs one permute and one FMA.  Otherwise q
// itself.
#ifndef RT_NODE_PRMT
#define RT_NODE_PRMT 1
#endif
#if RT_NODE_PRMT
constexpr float kQScale = 32768.0f;   // 2^15: one quantisation step per 2^-15
constexpr float kQOne = 1.0f;         // the byte's value at q = 0
#else
constexpr float kQScale = 1.0f;
constexpr float kQOne = 0.0f;
#endif
__device__ __forceinline__ float qbyte(uint32_t lo, uint32_t hi, int s)
{
#if RT_NODE_PRMT
    const uint32_t w = (s < 4) ? lo : hi;
    return __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u | ((uint32_t)(s & 3) << 4)));
#else
    return (float)byte_of(lo, hi, s);
#endif
}

// max / min of three floats (one instruction with RT_NODE_MINMAX3).
#ifndef RT_NODE_MINMAX3
#define RT_NODE_MINMAX3 1
#endif
__device__ __forceinline__ float fmax3f(float a, float b, float c)
{
#if RT_NODE_MINMAX3
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
#else
    return fmaxf(fmaxf(a, b), c);
#endif
}
__device__ __forceinline__ float fmin3f(float a, float b, float c)
{
#if RT_NODE_MINMAX3
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
#else
    return fminf(fminf(a, b), c);
#endif
}

// Packed single-precision FMA (fma.rn.f32x2, sm_100 family): two plane
// distances per instruction, each half rounded exactly as fmaf, so the
// child-box test and the frames are the same either way (measured faster:
// terrain frame -0.9 %, AO-instances frame -4.7 %).
#ifndef RT_NODE_FMA2
#define RT_NODE_FMA2 1
#endif
__device__ __forceinline__ uint64_t pack2f(float a, float b)
{
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 fma2f(float a0, float a1, uint64_t b, uint64_t c)
{
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pack2f(a0, a1)), "l"(b), "l"(c));
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(d));
    return r;
}

__device__ __forceinline__ NodeHits intersect_node(const WideNode *__restrict__ nodes, uint32_t idx, const float3 o,
                                                   const float3 inv, uint32_t oct, float tmax)
{
    const float4 *np = reinterpret_cast<const float4 *>(nodes + idx);
    const float4 n0 = __ldg(np + 0);
    const float4 n1 = __ldg(np + 1);
    const float4 n2 = __ldg(np + 2);
    const float4 n3 = __ldg(np + 3);
    const float4 n4 = __ldg(np + 4);
    const uint32_t e_imask = __float_as_uint(n0.w);
    const uint32_t ex = e_imask & 0xffu, ey = (e_imask >> 8) & 0xffu, ez = (e_imask >> 16) & 0xffu;
    const uint32_t imask = e_imask >> 24;
    // plane t = q * step + (origin - o) * inv, evaluated as
    // qbyte * (step * kQScale) + ((origin - o) * inv - kQOne * step * kQScale):
    // the folded offset rounds at the magnitude of 2^15 steps, an error below
    // 2^-9 of one step, far inside the one-step padding of every box
    const float ux = __uint_as_float(ex << 23) * inv.x;
    const float uy = __uint_as_float(ey << 23) * inv.y;
    const float uz = __uint_as_float(ez << 23) * inv.z;
    const float sx = ux * kQScale, sy = uy * kQScale, sz = uz * kQScale;
    const float ox = fmaf(-kQOne, sx, (n0.x - o.x) * inv.x);
    const float oy = fmaf(-kQOne, sy, (n0.y - o.y) * inv.y);
    const float oz = fmaf(-kQOne, sz, (n0.z - o.z) * inv.z);
    const uint32_t meta_lo = __float_as_uint(n1.z), meta_hi = __float_as_uint(n1.w);
    // lo/hi byte planes; swap per axis so "near" is the entry plane
    uint32_t nxl = __float_as_uint(n2.x), nxh = __float_as_uint(n2.y);   // qlo_x
    uint32_t nyl = __float_as_uint(n2.z), nyh = __float_as_uint(n2.w);   // qlo_y
    uint32_t nzl = __float_as_uint(n3.x), nzh = __float_as_uint(n3.y);   // qlo_z
    uint32_t fxl = __float_as_uint(n3.z), fxh = __float_as_uint(n3.w);   // qhi_x
    uint32_t fyl = __float_as_uint(n4.x), fyh = __float_as_uint(n4.y);   // qhi_y
    uint32_t fzl = __float_as_uint(n4.z), fzh = __float_as_uint(n4.w);   // qhi_z
    if (inv.x < 0.f) { uint32_t t = nxl; nxl = fxl; fxl = t; t = nxh; nxh = fxh; fxh = t; }
    if (inv.y < 0.f) { uint32_t t = nyl; nyl = fyl; fyl = t; t = nyh; nyh = fyh; fyh = t; }
    if (inv.z < 0.f) { uint32_t t = nzl; nzl = fzl; fzl = t; t = nzh; nzh = fzh; fzh = t; }
    uint32_t hits_int = 0, hits_tri = 0;
    // slot s with its six plane distances: internal children set bit
    // 24 + (s ^ oct), leaf slots their triangle bits.  An empty slot needs
    // no test of its meta byte: its box is inverted (low planes 255, high
    // planes 0), and should rounding let it "hit", its clear internal bit
    // and meta byte 0 add nothing.
    auto slot = [&](int s, float tnx, float tny, float tnz, float tfx, float tfy, float tfz) {
        const uint32_t meta = byte_of(meta_lo, meta_hi, s);
        const float tn = fmax3f(tnx, tny, fmaxf(tnz, 0.0f));
        const float tf = fmin3f(tfx, tfy, fminf(tfz, tmax));
        if (tn <= tf) {
            if ((imask >> s) & 1u) hits_int |= 1u << (24 + (s ^ oct));
            else hits_tri |= (meta >> 5) << (meta & 31u);
        }
    };
#if RT_NODE_FMA2
    const uint64_t SX = pack2f(sx, sx), SY = pack2f(sy, sy), SZ = pack2f(sz, sz);
    const uint64_t OX = pack2f(ox, ox), OY = pack2f(oy, oy), OZ = pack2f(oz, oz);
#pragma unroll
    for (int s = 0; s < 8; s += 2) {
        const float2 tnx = fma2f(qbyte(nxl, nxh, s), qbyte(nxl, nxh, s + 1), SX, OX);
        const float2 tny = fma2f(qbyte(nyl, nyh, s), qbyte(nyl, nyh, s + 1), SY, OY);
        const float2 tnz = fma2f(qbyte(nzl, nzh, s), qbyte(nzl, nzh, s + 1), SZ, OZ);
        const float2 tfx = fma2f(qbyte(fxl, fxh, s), qbyte(fxl, fxh, s + 1), SX, OX);
        const float2 tfy = fma2f(qbyte(fyl, fyh, s), qbyte(fyl, fyh, s + 1), SY, OY);
        const float2 tfz = fma2f(qbyte(fzl, fzh, s), qbyte(fzl, fzh, s + 1), SZ, OZ);
        slot(s, tnx.x, tny.x, tnz.x, tfx.x, tfy.x, tfz.x);
        slot(s + 1, tnx.y, tny.y, tnz.y, tfx.y, tfy.y, tfz.y);
    }
#else
#pragma unroll
    for (int s = 0; s < 8; ++s)
        slot(s, fmaf(qbyte(nxl, nxh, s), sx, ox), fmaf(qbyte(nyl, nyh, s), sy, oy), fmaf(qbyte(nzl, nzh, s), sz, oz),
             fmaf(qbyte(fxl, fxh, s), sx, ox), fmaf(qbyte(fyl, fyh, s), sy, oy), fmaf(qbyte(fzl, fzh, s), sz, oz));
#endif
    NodeHits h;
    h.ngroup = make_uint2(__float_as_uint(n1.x), hits_int | imask);
    h.tgroup = make_uint2(__float_as_uint(n1.y), hits_tri);
    return h;
}

__device__ __forceinline__ float3 safe_inv(float3 d)
{
    const float tiny = 1e-20f;
    const float x = (fabsf(d.x) > tiny) ? d.x : copysignf(tiny, d.x);
    const float y = (fabsf(d.y) > tiny) ? d.y : copysignf(tiny, d.y);
    const float z = (fabsf(d.z) > tiny) ? d.z : copysignf(tiny, d.z);
    return make_float3(__frcp_rn(x), __frcp_rn(y), __frcp_rn(z));
}

__device__ __forceinline__ uint32_t octant_of(float3 d)
{
    return (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
}

struct HitRecord {
    int32_t id;
    float t, u, v;
};
struct FetchCount {
    uint32_t nodes = 0;
    uint32_t tris = 0;
};

// Resumable traversal state of one ray: trav_begin sets it up, each
// trav_step intersects one node (or resumes a stacked node group) and tests
// that node's leaf triangles.  The stack lives with the caller.
struct Trav {
    float3 o, d, inv;
    uint32_t oct;
    float tmax;        // any-hit limit
    float box_tmax;    // boxes beyond this are culled (closest: best t so far)
    uint2 ngroup;
    int sp;
    int steps;
    HitRecord hit;
    bool occluded;
};

__device__ __forceinline__ void trav_begin(Trav &T, const SceneView &sc, const float3 o, const float3 d, float tmax,
                                           bool any)
{
    T.o = o;
    T.d = d;
    T.inv = safe_inv(d);
    T.oct = octant_of(d);
    T.tmax = tmax;
    T.box_tmax = any ? tmax : FLT_MAX;
    // a group holding only the root (as slot 0 of a virtual parent)
    T.ngroup = make_uint2((uint32_t)sc.root, sc.nnodes > 0 ? ((1u << (24 + T.oct)) | 1u) : 0u);
    T.sp = 0;
    T.steps = 0;
    T.hit.id = -1;
    T.hit.t = FLT_MAX;
    T.hit.u = 0.f;
    T.hit.v = 0.f;
    T.occluded = false;
}

// One traversal step; returns true when the ray is finished.  Closest hit
// (any = false) or any hit inside (EPSILON, tmax) skipping light and
// transparent triangles (any = true).  Status bits go to `status`.  STACK:
// the stack's capacity in node groups (a ray holds at most one group per
// tree level, so any capacity above the tree's depth suffices).
template <bool COUNT, int STACK = kStackSize>
__device__ __forceinline__ bool trav_step(Trav &T, uint2 *stack, const SceneView &sc, bool any, uint32_t &status,
                                          FetchCount *fc)
{
    if (++T.steps > kMaxTraversalSteps) { status |= kStatusStepLimit; return true; }
    uint2 tgroup = make_uint2(0u, 0u);
    if (T.ngroup.y & 0xff000000u) {
        const uint32_t bit = __ffs(T.ngroup.y >> 24) - 1u;
        T.ngroup.y &= ~(1u << (24 + bit));
        const uint32_t slot = bit ^ T.oct;
        const uint32_t idx = T.ngroup.x + __popc(T.ngroup.y & ((1u << slot) - 1u) & 0xffu);
        if (idx >= (uint32_t)sc.nnodes) { status |= kStatusBadIndex; return true; }
        if (T.ngroup.y & 0xff000000u) {
            if (T.sp >= STACK) { status |= kStatusStackOverflow; return true; }
            stack[T.sp++] = T.ngroup;
        }
        const NodeHits nh = intersect_node(sc.nodes, idx, T.o, T.inv, T.oct, T.box_tmax);
        if (COUNT) ++fc->nodes;
        T.ngroup = nh.ngroup;
        tgroup = nh.tgroup;
    }
    const bool watertight = sc.isect == RT_ISECT_WATERTIGHT;
    while (tgroup.y != 0u) {
        const uint32_t k = __ffs(tgroup.y) - 1u;
        tgroup.y &= tgroup.y - 1u;
        const uint32_t ti = tgroup.x + k;
        if (ti >= (uint32_t)sc.ntris) { status |= kStatusBadIndex; continue; }
        const PackedTri *tp = sc.tris + ti;
        if (COUNT) ++fc->tris;
        const float4 w0 = __ldg(&tp->w0);
        const float4 w1 = __ldg(&tp->w1);
        const float4 w2 = __ldg(&tp->w2);
        float u, v;
        const float t = watertight ? wt_intersect_ray(w0, w1, w2, T.o, T.d, &u, &v)
                                   : mt_intersect(w0, w1, w2, T.o, T.d, u, v);
        const int32_t id = __float_as_int(w2.y);
        if ((uint32_t)id >= (uint32_t)sc.ntris) { status |= kStatusBadIndex; continue; }
        if (any) {
            if ((__float_as_uint(w2.z) & (RT_TRI_LIGHT | RT_TRI_TRANSPARENT)) == 0u && t > kEpsilon && t < T.tmax) {
                T.occluded = true;
                T.hit.id = id;
                T.hit.t = t;
                return true;
            }
        } else if (t > kEpsilon && (t < T.hit.t || (t == T.hit.t && id < T.hit.id))) {
            T.hit.id = id;
            T.hit.t = t;
            T.hit.u = u;
            T.hit.v = v;
            T.box_tmax = t;
        }
    }
    if (!(T.ngroup.y & 0xff000000u)) {
        if (T.sp == 0) return true;
        T.ngroup = stack[--T.sp];
    }
    return false;
}

// Whole traversal of one ray.  Returns the device status bits.
template <bool ANY, bool COUNT = false, int STACK = kStackSize>
__device__ __forceinline__ uint32_t traverse(const SceneView &sc, const float3 o, const float3 d, float tmax,
                                             HitRecord &hit, bool &occluded, FetchCount *fc = nullptr)
{
    uint2 stack[STACK];
    Trav T;
    trav_begin(T, sc, o, d, tmax, ANY);
    uint32_t status = 0u;
    while (!trav_step<COUNT, STACK>(T, stack, sc, ANY, status, fc)) {
    }
    hit = T.hit;
    occluded = T.occluded;
    return status;
}

// ------------------------------------------------------------ shading

// ray::offset_start_point(d) (raytracer/ray.h:111-157) for d = +1 (out of
// the surface, dsign 1) or -1 (into it, the refraction start point): each
// coordinate moves by int(+-32 * n * d) units in the last place, or, when
// the coordinate is tiny, to 1e-4 * n whatever d.
__device__ __forceinline__ float offset_coord(float p, float n, float dsign = 1.0f)
{
    uint32_t x = __float_as_uint(p);
    if ((x & 0x7fffffffu) < 0x38d1b717u)   // bit pattern of 1.0e-4f
        return xadd(0.0f, xmul(1.0e-4f, n));
    const float off = ((x >> 31) & 1u) ? -32.0f : 32.0f;
    const float f = xmul(xmul(off, n), dsign);
    int32_t iv;
    if (!(f > -2147483904.0f && f < 2147483648.0f)) iv = INT32_MIN;
    else iv = __float2int_rz(f);
    x += (uint32_t)iv;
    return __uint_as_float(x);
}

__device__ __forceinline__ float3 offset_start(float3 p, float3 n)
{
    return make_float3(offset_coord(p.x, n.x), offset_coord(p.y, n.y), offset_coord(p.z, n.z));
}

__device__ __forceinline__ float3 offset_start_in(float3 p, float3 n)
{
    return make_float3(offset_coord(p.x, n.x, -1.0f), offset_coord(p.y, n.y, -1.0f), offset_coord(p.z, n.z, -1.0f));
}

// Camera ray of pixel (x, y) (camera.h:127-140, EXACT_NORMALISE).
__device__ __forceinline__ RayState camera_ray(const CameraView &cam, int x, int y)
{
    const float x_t = xadd(xmul((float)x, cam.x_inc), cam.x_m);
    const float y_t = xadd(xmul((float)y, cam.y_inc), cam.y_m);
    const float3 screen = xadd3(xadd3(xmul3(cam.X, x_t), xmul3(cam.Y, y_t)), xmul3(cam.Z, cam.t));
    RayState r;
    r.o = cam.c;
    r.d = xnorm(screen);
    return r;
}

struct SurfacePoint {
    float3 dst;       // refined hit point
    float3 sn;        // face-forwarded shading normal
    float3 geo;       // face-forwarded geometric normal
    float3 vt;        // interpolated per-vertex attribute
    bool has_attr;
    bool out_in;      // the ray meets the front face (hit_t::out_in)
};

// Hit refinement and face-forwarding (raytracer.cc:30-31,
// triangle::normal_at_point triangle.h:464-498) and the barycentric
// attribute (triangle.h:74-79).
__device__ __forceinline__ SurfacePoint surface_at(const SceneView &sc, const RayState &r, const HitRecord &h)
{
    SurfacePoint sp;
    const ShadeTri st = sc.shade[h.id];
    const float3 n = make_float3(st.n_cx.x, st.n_cx.y, st.n_cx.z);
    const float3 c = make_float3(st.n_cx.w, st.c_yz.x, st.c_yz.y);
    float3 p = xadd3(r.o, xmul3(r.d, h.t));
    const float denom = xdot(n, r.d);
    const float num = xdot(n, xsub3(c, p));
    p = xadd3(p, xmul3(r.d, xdiv(num, denom)));
    // shading normal: the triangle's corner normals interpolated by the
    // hit's barycentrics when it has them (triangle.h:473-476), else the
    // face normal; both face-forwarded with the face normal's test
    float3 sn = n;
    if (sc.cnorm) {
        const float *cn = sc.cnorm + 9 * (size_t)h.id;
        if (cn[0] != FLT_MAX) {
            const float3 A = make_float3(cn[0], cn[1], cn[2]), B = make_float3(cn[3], cn[4], cn[5]),
                         C = make_float3(cn[6], cn[7], cn[8]);
            const float w = xsub(1.0f, xadd(h.u, h.v));
            sn = xadd3(xadd3(xmul3(C, h.u), xmul3(B, h.v)), xmul3(A, w));
        }
    }
    if (denom > 0.0f) {
        sp.sn = make_float3(-sn.x, -sn.y, -sn.z);
        sp.geo = make_float3(-n.x, -n.y, -n.z);
    } else {
        sp.sn = sn;
        sp.geo = n;
    }
    sp.out_in = !(denom > 0.0f);
    sp.dst = p;
    sp.has_attr = sc.vattr != nullptr;
    if (sp.has_attr) {
        const int3 t = sc.idx[h.id];
        const float3 A = make_float3(sc.vattr[3 * t.x], sc.vattr[3 * t.x + 1], sc.vattr[3 * t.x + 2]);
        const float3 B = make_float3(sc.vattr[3 * t.y], sc.vattr[3 * t.y + 1], sc.vattr[3 * t.y + 2]);
        const float3 C = make_float3(sc.vattr[3 * t.z], sc.vattr[3 * t.z + 1], sc.vattr[3 * t.z + 2]);
        const float w = xsub(1.0f, xadd(h.u, h.v));
        sp.vt = xadd3(xadd3(xmul3(C, h.u), xmul3(B, h.v)), xmul3(A, w));
    } else {
        sp.vt = make_float3(FLT_MAX, FLT_MAX, FLT_MAX);
    }
    return sp;
}

// Diffuse colour (coloured_mapper_shader.cc:61-66 with attribute*255 samples).
__device__ __forceinline__ float3 material_kd(const MaterialView &m, const SurfacePoint &sp)
{
    if (!sp.has_attr || (m.flags & RT_MAT_NO_VERTEX_COLOUR)) return m.kd;
    const float k = 1.0f / 255.0f;
    return make_float3(xmul(xmul(sp.vt.x, 255.0f), xmul(m.kd.x, k)), xmul(xmul(sp.vt.y, 255.0f), xmul(m.kd.y, k)),
                       xmul(xmul(sp.vt.z, 255.0f), xmul(m.kd.z, k)));
}

// Shadow ray towards a light (ray::find_rays ray.cc:91-104,
// light::find_rays light.h:62-100, ray::set_up ray.h:44-54).
__device__ __forceinline__ void shadow_ray(const LightView &L, float3 start, float3 &dir, float &len)
{
    const float3 target = (L.kind == RT_LIGHT_DIRECTIONAL) ? xadd3(start, xmul3(L.dir, L.dist_sign)) : L.pos;
    const float3 dv = xsub3(target, start);
    len = xmag(dv);
    dir = xdiv3(dv, len);
}

// One light's Phong term (coloured_mapper_shader.cc:76-109,
// light::get_light_intensity light.h:44-59) added into c.  EXACT = true
// evaluates the specular power in double and rounds once, the reference's
// result; EXACT = false uses single-precision powf (a few ulp), whose frames
// are made exact by exact_if_near_boundary below.
template <bool EXACT = true>
__device__ __forceinline__ void phong_add(const LightView &L, const MaterialView &m, const float3 kd, const float3 sn,
                                          const float3 view_dir, const float3 ldir, float len, float magn, float3 &c)
{
    const float shade = xdot(ldir, sn);
    if (shade < 0.0f) return;
    const float3 ref = xsub3(ldir, xmul3(sn, xmul(2.0f, shade)));
    const float rdr = xdot(view_dir, ref);
    float3 sc = make_float3(xmul(shade, kd.x), xmul(shade, kd.y), xmul(shade, kd.z));
    if (rdr > 0.0f) {
        const float p = EXACT ? (float)pow((double)rdr, (double)m.ns) : powf(rdr, m.ns);
        sc = make_float3(xadd(sc.x, xmul(p, m.ks.x)), xadd(sc.y, xmul(p, m.ks.y)), xadd(sc.z, xmul(p, m.ks.z)));
    }
    const float dist = xmul(len, L.d);
    const float d_scale = xadd(xmul(dist, dist), 1.0f);
    float3 I;
    if (L.s_b != 0.0f) {
        // spot light: intensity by the angle off its axis (light.h:49-55);
        // the angle always in double, rounded once: divided by a narrow
        // cone width, a few ulp of acosf would not stay within the
        // truncation guard
        const float cosa = xdot(ldir, L.dir);
        const float a = (float)acos((double)cosa);
        const float p = xdiv(xsub(a, L.s_a), xsub(L.s_b, L.s_a));
        const float q = xsub(1.0f, p);
        const float f = (0.0f < ((q < 1.0f) ? q : 1.0f)) ? ((q < 1.0f) ? q : 1.0f) : 0.0f;   // max(0, min(1, q))
        const float fs = xdiv(f, d_scale);
        I = make_float3(xmul(L.rgb255.x, fs), xmul(L.rgb255.y, fs), xmul(L.rgb255.z, fs));
    } else {
        I = make_float3(xdiv(L.rgb255.x, d_scale), xdiv(L.rgb255.y, d_scale), xdiv(L.rgb255.z, d_scale));
    }
    c = make_float3(xadd(c.x, xmul(I.x, xmul(sc.x, magn))), xadd(c.y, xmul(I.y, xmul(sc.y, magn))),
                    xadd(c.z, xmul(I.z, xmul(sc.z, magn))));
}

// camera::clip_image_to_rgb (camera.h:312-314): clamp, then truncate.
__device__ __forceinline__ uint8_t clip8(float v)
{
    return (uint8_t)__float2uint_rz(smin(255.0f, smax(0.0f, xdiv(v, 1.0f))));
}

// The single-precision specular power differs from the exact one by a few
// ulp (<= 1e-6 relative), which moves a colour channel by far less than
// kTruncGuard; only a channel that close to an integer can truncate
// differently.
constexpr float kTruncGuard = 4e-3f;
__device__ __forceinline__ bool near_integer(float v)
{
    const float f = v - floorf(v);
    return f < kTruncGuard || f > 1.0f - kTruncGuard;
}
__device__ __forceinline__ bool near_truncation(float3 c)
{
    return near_integer(c.x) || near_integer(c.y) || near_integer(c.z);
}

// Colour of a hit pixel with the exact specular power, from the stored
// shading inputs and per-light shadow answers (bit l = light l blocked).
__device__ __forceinline__ float3 shade_lights_exact(const LightView *lights, int nl, const MaterialView &mat,
                                                     float3 kd, float3 sn, float3 view_dir, float3 start,
                                                     uint32_t blocked_bits)
{
    float3 c = make_float3(0.f, 0.f, 0.f);
    for (int l = 0; l < nl; ++l) {
        float3 ldir;
        float len;
        shadow_ray(lights[l], start, ldir, len);
        phong_add<true>(lights[l], mat, kd, sn, view_dir, ldir, len, ((blocked_bits >> l) & 1u) ? 0.0f : 1.0f, c);
    }
    return xadd3(c, mat.ka);
}

// ---------------------------------------------------------- AO sampler

// Philox4x32-10 (Salmon et al., SC'11).
__device__ __forceinline__ uint4 philox4x32(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

struct AOBasis {
    float3 T, B, g;
};

// Orthonormal basis of Duff et al. (JCGT 2017), IEEE-exact.
__device__ __forceinline__ AOBasis ao_basis(float3 g)
{
    const float sign = (g.z < 0.0f || (g.z == 0.0f && (__float_as_uint(g.z) >> 31))) ? -1.0f : 1.0f;
    const float a = xdiv(-1.0f, xadd(sign, g.z));
    const float b = xmul(xmul(g.x, g.y), a);
    AOBasis ob;
    ob.T = make_float3(xadd(1.0f, xmul(xmul(sign, xmul(g.x, g.x)), a)), xmul(sign, b), -xmul(sign, g.x));
    ob.B = make_float3(b, xadd(sign, xmul(xmul(g.y, g.y), a)), -g.y);
    ob.g = g;
    return ob;
}

// Direction of AO sample s for a pixel (cosine-weighted by rejection from
// the unit disk, at most 8 tries, lifted to the hemisphere).
__device__ __forceinline__ float3 ao_direction(const AOBasis &ob, uint32_t pixel, uint32_t s, uint32_t seed)
{
    float x = 0.0f, y = 0.0f;
    bool found = false;
    for (uint32_t call = 0; call < 4 && !found; ++call) {
        const uint4 r = philox4x32(make_uint4(pixel, s, call, 0x414f5259u), seed, 0x52415054u);
        const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
        for (int pair = 0; pair < 2; ++pair) {
            if (found) break;
            const float px = xsub(xmul((float)(rr[2 * pair] >> 8), 1.1920928955078125e-7f), 1.0f);
            const float py = xsub(xmul((float)(rr[2 * pair + 1] >> 8), 1.1920928955078125e-7f), 1.0f);
            if (xadd(xmul(px, px), xmul(py, py)) < 1.0f) { x = px; y = py; found = true; }
        }
    }
    const float z = __fsqrt_rn(smax(0.0f, xsub(1.0f, xadd(xmul(x, x), xmul(y, y)))));
    const float3 d = xadd3(xadd3(xmul3(ob.T, x), xmul3(ob.B, y)), xmul3(ob.g, z));
    return xnorm(d);
}

}  // namespace rtc
