// rt_adjoint.cu -- differentiable rendering: float forward and the
// hand-written adjoint of the primary+shadow Phong frame.
//
// Forward model of a pixel whose primary ray hits triangle (a, b, c)
// (visibility and the hit triangle held fixed, interior gradients only):
//   o + t d = (1-u-v) a + v b + u c          (u weighs c, v weighs b)
//   n  = normalize((b-a) x (c-a)),  sn = +-n  (faces the viewer)
//   col = u C_c + v C_b + (1-u-v) C_a        (per-vertex colour)
//   per light: L = (P - p)/|P - p| (point) or the fixed direction,
//   s = L.sn, r = d.(L - 2 s sn), I = rgb/255 / ((|P-p| D)^2 + 1),
//   pix += vis I (s kd col + [r > 0] r^ns ks)   when s >= 0
//   pix += ka
// The adjoint kernel re-traces the pixel's primary and shadow rays (so the
// only per-pixel storage is dL/dpixel), back-propagates dL/dpix through the
// shading, the normal, the light vector and the ray-triangle solve, and
// scatters dL/dposition and dL/dcolour onto the triangle's vertices with
// atomics.  Memory is O(pixels + vertices).
#include "rt_api_internal.cuh"
#include "rt_shade.cuh"

using namespace rtc;

namespace rtc {
namespace {

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double3 cross3d(double3 a, double3 b)
{
    return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ void atomic_add3(float *p, float3 g)
{
    atomicAdd(p, g.x);
    atomicAdd(p + 1, g.y);
    atomicAdd(p + 2, g.z);
}

template <bool ADJOINT>
__global__ void __launch_bounds__(kTraceThreads) k_diff(SceneView sc, const float *__restrict__ verts,
                                                        CameraView cam, LightSet lights, MaterialView mat,
                                                        float *__restrict__ fimg, int32_t *__restrict__ ids,
                                                        uint8_t *__restrict__ occl, const float *__restrict__ dldpix,
                                                        float *__restrict__ gpos,
                                                        float *__restrict__ gcol, Counters *ctr)
{
    int tiles_x;
    const int items = tiles_of<8>(cam.xres, cam.yres, tiles_x) * 32;
    uint32_t status = 0;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel<8>(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
        bool hit = false;
        uint32_t nsec = 0;
        if (live) {
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            const RayState r = camera_ray(cam, x, y);
            HitRecord h;
            bool occ;
            status |= traverse<false>(sc, r.o, r.d, FLT_MAX, h, occ);
            hit = h.t < FLT_MAX;
            if (!ADJOINT) {
                // float forward: the same per-pixel work as rt_render, unclipped
                float3 c = cam.background;
                uint32_t obits = 0;
                if (hit) {
                    const SurfacePoint sp = surface_at(sc, r, h);
                    const float3 start = offset_start(sp.dst, sp.geo);
                    const float3 kd = material_kd(mat, sp);
                    c = make_float3(0.f, 0.f, 0.f);
                    for (int l = 0; l < lights.n; ++l) {
                        float3 ldir;
                        float len;
                        shadow_ray(lights.l[l], start, ldir, len);
                        HitRecord sh;
                        bool blocked;
                        status |= traverse<true>(sc, start, ldir, len, sh, blocked);
                        ++nsec;
                        if (blocked) obits |= 1u << l;
                        phong_add(lights.l[l], mat, kd, sp.sn, r.d, ldir, len, blocked ? 0.0f : 1.0f, c);
                    }
                    c = xadd3(c, mat.ka);
                }
                fimg[3 * pix] = c.x;
                fimg[3 * pix + 1] = c.y;
                fimg[3 * pix + 2] = c.z;
                if (ids) ids[pix] = hit ? h.id : -1;
                if (occl) occl[pix] = (uint8_t)obits;
            } else if (hit) {
                const float3 g = f3(dldpix[3 * pix], dldpix[3 * pix + 1], dldpix[3 * pix + 2]);
                const SurfacePoint sp = surface_at(sc, r, h);
                const float3 start = offset_start(sp.dst, sp.geo);
                const int3 tv = sc.idx[h.id];
                const float3 A = f3(verts[3 * tv.x], verts[3 * tv.x + 1], verts[3 * tv.x + 2]);
                const float3 B = f3(verts[3 * tv.y], verts[3 * tv.y + 1], verts[3 * tv.y + 2]);
                const float3 Cv = f3(verts[3 * tv.z], verts[3 * tv.z + 1], verts[3 * tv.z + 2]);
                const float u = h.u, v = h.v, w = 1.0f - u - v;
                const float3 d = r.d;
                const float3 p = r.o + d * h.t;
                // normal and its orientation
                const float3 e2 = B - A, e1 = Cv - A;
                const float3 m = cross3(e2, e1);
                const float mlen = sqrtf(dot3(m, m));
                const float3 n = m * (1.0f / mlen);
                const float sgn = (dot3(n, d) > 0.0f) ? -1.0f : 1.0f;
                const float3 sn = n * sgn;
                // colour
                float3 col = mat.kd, cA = f3(0, 0, 0), cB = f3(0, 0, 0), cC = f3(0, 0, 0);
                const bool attr = sc.vattr != nullptr;
                if (attr) {
                    cA = f3(sc.vattr[3 * tv.x], sc.vattr[3 * tv.x + 1], sc.vattr[3 * tv.x + 2]);
                    cB = f3(sc.vattr[3 * tv.y], sc.vattr[3 * tv.y + 1], sc.vattr[3 * tv.y + 2]);
                    cC = f3(sc.vattr[3 * tv.z], sc.vattr[3 * tv.z + 1], sc.vattr[3 * tv.z + 2]);
                    const float3 vt = cC * u + cB * v + cA * w;
                    col = f3(vt.x * mat.kd.x, vt.y * mat.kd.y, vt.z * mat.kd.z);
                }
                float3 g_p = f3(0, 0, 0), g_sn = f3(0, 0, 0), g_col = f3(0, 0, 0);
                for (int l = 0; l < lights.n; ++l) {
                    const LightView &L = lights.l[l];
                    float3 ldir_f;
                    float len_f;
                    shadow_ray(L, start, ldir_f, len_f);
                    HitRecord sh;
                    bool blocked;
                    status |= traverse<true>(sc, start, ldir_f, len_f, sh, blocked);
                    ++nsec;
                    if (blocked) continue;
                    // analytic light vector from the unrefined hit point
                    float3 ldir;
                    float len;
                    const bool point = L.kind != RT_LIGHT_DIRECTIONAL;
                    if (point) {
                        const float3 wv = L.pos - p;
                        len = sqrtf(dot3(wv, wv));
                        ldir = wv * (1.0f / len);
                    } else {
                        ldir = ldir_f;
                        len = len_f;
                    }
                    const float s = dot3(ldir, sn);
                    if (s < 0.0f) continue;
                    const float dsn = dot3(d, sn);
                    const float rr = dot3(d, ldir) - 2.0f * s * dsn;
                    const float dist = len * L.d;
                    const float den = dist * dist + 1.0f;
                    const float3 I = f3(L.rgb255.x / den, L.rgb255.y / den, L.rgb255.z / den);
                    float S = 0.0f, dS = 0.0f;
                    if (rr > 0.0f) {
                        S = powf(rr, mat.ns);
                        dS = (mat.ns != 0.0f) ? mat.ns * powf(rr, mat.ns - 1.0f) : 0.0f;
                    }
                    // upstream of this light's term  I * (s col + S ks)
                    const float3 term = f3(s * col.x + S * mat.ks.x, s * col.y + S * mat.ks.y, s * col.z + S * mat.ks.z);
                    // sum_c g_c I_c term_c: the upstream of the common 1/den factor
                    const float gI = g.x * I.x * term.x + g.y * I.y * term.y + g.z * I.z * term.z;
                    const float g_s = g.x * I.x * col.x + g.y * I.y * col.y + g.z * I.z * col.z;
                    const float g_S = g.x * I.x * mat.ks.x + g.y * I.y * mat.ks.y + g.z * I.z * mat.ks.z;
                    g_col = g_col + f3(g.x * I.x * s, g.y * I.y * s, g.z * I.z * s);
                    const float g_r = g_S * dS;
                    const float g_s_tot = g_s + g_r * (-2.0f * dsn);
                    float3 g_ldir = d * g_r + sn * g_s_tot;
                    g_sn = g_sn + ldir * g_s_tot + d * (g_r * (-2.0f * s));
                    if (point) {
                        // I_c = rgb_c / den, den = (len D)^2 + 1: dI_c/dlen = -I_c 2 len D^2 / den
                        const float g_len = -gI * (2.0f * len * L.d * L.d / den);
                        // ldir = wv / len, len = |wv|, wv = P - p
                        const float3 g_wv = (g_ldir - ldir * dot3(g_ldir, ldir)) * (1.0f / len) + ldir * g_len;
                        g_p = g_p - g_wv;
                    }
                }
                // normal: sn = sgn m/|m|, m = e2 x e1
                const float3 g_n = g_sn * sgn;
                const float3 g_m = (g_n - n * dot3(g_n, n)) * (1.0f / mlen);
                float3 gA = f3(0, 0, 0), gB = f3(0, 0, 0), gC = f3(0, 0, 0);
                // m = X x Y, X = e2 = B - A, Y = e1 = C - A
                const float3 gX = cross3(e1, g_m);   // dL/dX = Y x g_m
                const float3 gY = cross3(g_m, e2);   // dL/dY = g_m x X
                gB = gB + gX;
                gC = gC + gY;
                gA = gA - gX - gY;
                // colour interpolation -> u, v and vertex colours
                float g_u = 0.0f, g_v = 0.0f;
                if (attr) {
                    const float3 gc = f3(g_col.x * mat.kd.x, g_col.y * mat.kd.y, g_col.z * mat.kd.z);
                    g_u = dot3(gc, cC - cA);
                    g_v = dot3(gc, cB - cA);
                    atomic_add3(gcol + 3 * tv.z, gc * u);
                    atomic_add3(gcol + 3 * tv.y, gc * v);
                    atomic_add3(gcol + 3 * tv.x, gc * w);
                }
                // ray-triangle solve: rows d, -e1, -e2 of M^T; lambda = M^-T (g_t, g_u, g_v).
                // Its determinant d.(e1 x e2) shrinks with the grazing angle
                // d.n, which scales the rounding error of a binary32 solve by
                // 1/|d.n|; the solve is done in double (one per hit pixel).
                const float g_t = dot3(g_p, d);
                const double3 r0 = make_double3(d.x, d.y, d.z);
                const double3 r1 = make_double3(-(double)e1.x, -(double)e1.y, -(double)e1.z);
                const double3 r2 = make_double3(-(double)e2.x, -(double)e2.y, -(double)e2.z);
                const double3 c12 = cross3d(r1, r2), c20 = cross3d(r2, r0), c01 = cross3d(r0, r1);
                const double det = r0.x * c12.x + r0.y * c12.y + r0.z * c12.z;
                if (fabs(det) > 1e-300) {
                    const double inv = 1.0 / det;
                    const double gt = g_t, gu = g_u, gv = g_v;
                    const float3 lam = f3((float)((c12.x * gt + c20.x * gu + c01.x * gv) * inv),
                                          (float)((c12.y * gt + c20.y * gu + c01.y * gv) * inv),
                                          (float)((c12.z * gt + c20.z * gu + c01.z * gv) * inv));
                    gA = gA + lam * w;
                    gB = gB + lam * v;
                    gC = gC + lam * u;
                }
                atomic_add3(gpos + 3 * tv.x, gA);
                atomic_add3(gpos + 3 * tv.y, gB);
                atomic_add3(gpos + 3 * tv.z, gC);
            }
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, hit);
        warp_add(&ctr->secondary, nsec);
    }
    if (status) atomicOr(&ctr->status, status);
}

}  // namespace
}  // namespace rtc

namespace {

#define RT_CUDA_A(call, what)                                  \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return set_cuda_error(_e, what); \
    } while (0)

struct Guard {
    int prev = -1;
    explicit Guard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~Guard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// Resident blocks per SM of a kernel (asked once per kernel; the grid is
// this times the calling context's SM count).
template <typename K>
int blocks_per_sm(K kernel)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceThreads, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 4;
    }
    return per_sm;
}

rt_status check_frame(rt_scene *s, const rt_camera *cam, const rt_light *lights, int32_t nl, const rt_material *m)
{
    if (!s || !cam || !m) return set_error(RT_ERR_INVALID_ARG, "NULL argument");
    if (cam->xres <= 0 || cam->yres <= 0 || (int64_t)cam->xres * cam->yres > (int64_t)1 << 28)
        return set_error(RT_ERR_INVALID_ARG, "camera resolution out of range");
    if (nl < 0 || nl > RT_MAX_LIGHTS || (nl > 0 && !lights)) return set_error(RT_ERR_INVALID_ARG, "light count out of range");
    if (m->rf != 0.0f || m->tran != 0.0f)
        return set_error(RT_ERR_INVALID_ARG,
                         "reflective or transparent materials (rf, tran > 0) are rendered by rt_render only");
    for (int32_t i = 0; i < nl; ++i)
        if ((lights[i].kind & ~RT_LIGHT_UNIT_RGB) == RT_LIGHT_SPOT && lights[i].s_b != 0.0f)
            return set_error(RT_ERR_INVALID_ARG, "spot lights are not differentiated (rt_render renders them)");
    if (!s->built) return set_error(RT_ERR_NOT_BUILT, "hierarchy not built");
    return RT_OK;
}

rt_status finish(rt_context *ctx, rt_render_stats *stats)
{
    RT_CUDA_A(cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream),
              "counter readback");
    RT_CUDA_A(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    const Counters c = *ctx->h_counters;
    if (stats) {
        stats->primary_rays = (int64_t)c.primary;
        stats->secondary_rays = (int64_t)c.secondary;
        stats->primary_hits = (int64_t)c.hits;
        stats->status = (int32_t)c.status;
        stats->nodes_fetched = 0;
        stats->tris_tested = 0;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        stats->device_ms = ms;
    }
    return status_to_error(c.status);
}

}  // namespace

extern "C" {

rt_status rt_scene_update_attributes(rt_scene *s, const float *vattr, int32_t nverts)
{
    if (!s || !vattr) return set_error(RT_ERR_INVALID_ARG, "rt_scene_update_attributes: NULL argument");
    if (nverts != s->nverts) return set_error(RT_ERR_INVALID_ARG, "rt_scene_update_attributes: vertex count changed");
    Guard g(s->ctx->device);
    const size_t bytes = (size_t)(nverts > 0 ? nverts : 1) * 3 * sizeof(float);
    if (!s->d_vattr) RT_CUDA_A(cudaMalloc(&s->d_vattr, bytes), "attribute allocation");
    if (nverts > 0)
        RT_CUDA_A(cudaMemcpyAsync(s->d_vattr, vattr, (size_t)nverts * 3 * sizeof(float), cudaMemcpyDefault, s->ctx->stream),
                  "attribute copy");
    RT_CUDA_A(cudaStreamSynchronize(s->ctx->stream), "attribute synchronize");
    return RT_OK;
}

rt_status rt_render_float(rt_scene *s, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                          const rt_material *material, float *rgb_f32, int32_t *hit_ids, uint8_t *occluded,
                          rt_render_stats *stats)
{
    rt_status st = check_frame(s, camera, lights, nlights, material);
    if (st != RT_OK) return st;
    if (!rgb_f32 || !is_device_ptr(rgb_f32) || (hit_ids && !is_device_ptr(hit_ids)) ||
        (occluded && !is_device_ptr(occluded)))
        return set_error(RT_ERR_INVALID_ARG, "rt_render_float: outputs must be device memory");
    rt_context *ctx = s->ctx;
    Guard g(ctx->device);
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = 0;
    for (int i = 0; i < nlights; ++i) ls.l[i] = make_light_view(lights[i]);
    static const int per_sm = blocks_per_sm(k_diff<false>);
    const int grid = per_sm * ctx->sm_count;
    RT_CUDA_A(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA_A(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    k_diff<false><<<grid, kTraceThreads, 0, ctx->stream>>>(scene_view(s), s->d_verts, make_camera_view(*camera), ls,
                                                           make_material_view(*material), rgb_f32, hit_ids, occluded,
                                                           nullptr, nullptr, nullptr, ctx->d_counters);
    RT_CUDA_A(cudaGetLastError(), "forward launch");
    RT_CUDA_A(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    return finish(ctx, stats);
}

rt_status rt_render_adjoint(rt_scene *s, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                            const rt_material *material, const float *dL_dpix, float *dL_dpos, float *dL_dattr,
                            rt_render_stats *stats)
{
    rt_status st = check_frame(s, camera, lights, nlights, material);
    if (st != RT_OK) return st;
    if (!dL_dpix || !dL_dpos || !dL_dattr || !is_device_ptr(dL_dpix) || !is_device_ptr(dL_dpos) ||
        !is_device_ptr(dL_dattr))
        return set_error(RT_ERR_INVALID_ARG, "rt_render_adjoint: buffers must be device memory");
    rt_context *ctx = s->ctx;
    Guard g(ctx->device);
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = 0;
    for (int i = 0; i < nlights; ++i) ls.l[i] = make_light_view(lights[i]);
    static const int per_sm = blocks_per_sm(k_diff<true>);
    const int grid = per_sm * ctx->sm_count;
    const size_t gbytes = (size_t)(s->nverts > 0 ? s->nverts : 1) * 3 * sizeof(float);
    RT_CUDA_A(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA_A(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    RT_CUDA_A(cudaMemsetAsync(dL_dpos, 0, gbytes, ctx->stream), "gradient clear");
    RT_CUDA_A(cudaMemsetAsync(dL_dattr, 0, gbytes, ctx->stream), "gradient clear");
    k_diff<true><<<grid, kTraceThreads, 0, ctx->stream>>>(scene_view(s), s->d_verts, make_camera_view(*camera), ls,
                                                          make_material_view(*material), nullptr, nullptr, nullptr,
                                                          dL_dpix, dL_dpos, dL_dattr, ctx->d_counters);
    RT_CUDA_A(cudaGetLastError(), "adjoint launch");
    RT_CUDA_A(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    return finish(ctx, stats);
}

}  // extern "C"
