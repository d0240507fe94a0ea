// rt_shade.cuh -- per-pixel work shared by the single-frame and batched
// render kernels (so both produce the same bits), and the warp-level helpers
// of the persistent kernels.
#pragma once

#include "rt_kernels.cuh"
#include "rt_traverse.cuh"

namespace rtc {

// Claim `chunk` consecutive work items for the whole warp.
__device__ __forceinline__ int warp_claim(int *counter, int chunk)
{
    int base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(counter, chunk);
    return __shfl_sync(0xffffffffu, base, 0);
}

__device__ __forceinline__ void warp_count(unsigned long long *ctr, bool pred)
{
    const uint32_t b = __ballot_sync(0xffffffffu, pred);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(ctr, (unsigned long long)__popc(b));
}

__device__ __forceinline__ void warp_add(unsigned long long *ctr, uint32_t v)
{
    uint32_t s = v;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(ctr, (unsigned long long)s);
}

// Pixel of work item `item`: tiles of TW x (32 / TW) pixels, one warp each.
template <int TW>
__device__ __forceinline__ void tile_pixel(int item, int tiles_x, int &x, int &y)
{
    constexpr int TH = 32 / TW;
    const int tile = item >> 5, lane = item & 31;
    x = (tile % tiles_x) * TW + (lane % TW);
    y = (tile / tiles_x) * TH + (lane / TW);
}

template <int TW>
__host__ __device__ __forceinline__ int tiles_of(int xres, int yres, int &tiles_x)
{
    constexpr int TH = 32 / TW;
    tiles_x = (xres + TW - 1) / TW;
    return tiles_x * ((yres + TH - 1) / TH);
}

struct PixelOut {
    float3 c;
    int32_t id;          // caller's triangle id, -1 on a miss
    bool hit;
    uint32_t secondary;  // shadow / AO rays traced
    int32_t ao_made;     // unoccluded AO rays
};

// Primary ray, closest hit, one shadow ray per light, coloured Phong
// (ray_trace_engine::ray_trace, raytracer.cc:20-87).
template <bool COUNT>
__device__ __forceinline__ PixelOut shade_pixel_lights(const SceneView &sc, const CameraView &cam, const LightView *lights,
                                                       int nl, const MaterialView &mat, int x, int y,
                                                       uint32_t &status, FetchCount *fc, bool fast_pow)
{
    PixelOut out;
    out.secondary = 0;
    out.ao_made = 0;
    const RayState r = camera_ray(cam, x, y);
    HitRecord h;
    bool occ;
    status |= traverse<false, COUNT>(sc, r.o, r.d, FLT_MAX, h, occ, fc);
    out.hit = h.t < FLT_MAX;
    out.id = out.hit ? h.id - sc.tri_base : -1;
    out.c = cam.background;
    if (out.hit) {
        const SurfacePoint sp = surface_at(sc, r, h);
        const float3 start = offset_start(sp.dst, sp.geo);
        const float3 kd = material_kd(mat, sp);
        float3 c = make_float3(0.f, 0.f, 0.f);
        uint32_t blocked_bits = 0;
        for (int l = 0; l < nl; ++l) {
            const LightView &L = lights[l];
            float3 ldir;
            float len;
            shadow_ray(L, start, ldir, len);
            HitRecord sh;
            bool blocked;
            status |= traverse<true, COUNT>(sc, start, ldir, len, sh, blocked, fc);
            ++out.secondary;
            if (blocked) blocked_bits |= 1u << l;
            if (fast_pow) phong_add<false>(L, mat, kd, sp.sn, r.d, ldir, len, blocked ? 0.0f : 1.0f, c);
            else phong_add<true>(L, mat, kd, sp.sn, r.d, ldir, len, blocked ? 0.0f : 1.0f, c);
        }
        out.c = xadd3(c, mat.ka);
        if (fast_pow && near_truncation(out.c))
            out.c = shade_lights_exact(lights, nl, mat, kd, sp.sn, r.d, start, blocked_bits);
    }
    return out;
}

// Primary ray and its chain of mirror reflections (reflective material,
// rf > 0): at every hit the coloured Phong of shade_pixel_lights with the
// exact specular power, then, while the ray's power magn * rf exceeds 0.1
// (compared in double, as the reference's MIN_REFLECTIVE_POWER literal), the
// mirror ray dir - n * (2 dir.n) from the offset start point (ray::reflect,
// ray.cc:118-135).  The colours combine from the deepest ray outwards,
// c_k + c_(k+1) * rf (combind_secondary_rays, coloured_mapper_shader.cc:
// 117-122); a ray that misses is the background.  `chain` holds up to
// RT_MAX_BOUNCES + 1 colours.
template <bool COUNT>
__device__ __forceinline__ PixelOut shade_pixel_reflect(const SceneView &sc, const CameraView &cam, const LightView *lights,
                                                        int nl, const MaterialView &mat, int x, int y, float3 *chain,
                                                        uint32_t &status, FetchCount *fc)
{
    PixelOut out;
    out.secondary = 0;
    out.ao_made = 0;
    out.hit = false;
    out.id = -1;
    RayState r = camera_ray(cam, x, y);
    float magn = 1.0f;
    int last = 0;
    for (int k = 0;; ++k) {
        HitRecord h;
        bool occ;
        status |= traverse<false, COUNT>(sc, r.o, r.d, FLT_MAX, h, occ, fc);
        if (k > 0) ++out.secondary;
        if (!(h.t < FLT_MAX)) {
            chain[k] = cam.background;
            last = k;
            break;
        }
        if (k == 0) {
            out.hit = true;
            out.id = h.id - sc.tri_base;
        }
        const SurfacePoint sp = surface_at(sc, r, h);
        const float3 start = offset_start(sp.dst, sp.geo);
        const float3 kd = material_kd(mat, sp);
        float3 c = make_float3(0.f, 0.f, 0.f);
        for (int l = 0; l < nl; ++l) {
            float3 ldir;
            float len;
            shadow_ray(lights[l], start, ldir, len);
            HitRecord sh;
            bool blocked;
            status |= traverse<true, COUNT>(sc, start, ldir, len, sh, blocked, fc);
            ++out.secondary;
            phong_add<true>(lights[l], mat, kd, sp.sn, r.d, ldir, len, blocked ? 0.0f : 1.0f, c);
        }
        chain[k] = xadd3(c, mat.ka);
        const float power = xmul(magn, mat.rf);
        if (!((double)power > 0.1) || k == RT_MAX_BOUNCES) {
            if ((double)power > 0.1) status |= kStatusStepLimit;   // deeper than the host allowed
            last = k;
            break;
        }
        const float rdn = xmul(2.0f, xdot(r.d, sp.sn));
        r.o = start;
        r.d = xsub3(r.d, xmul3(sp.sn, rdn));
        magn = power;
    }
    float3 acc = chain[last];
    for (int k = last - 1; k >= 0; --k) acc = xadd3(chain[k], xmul3(acc, mat.rf));
    out.c = acc;
    return out;
}

// Primary ray, closest hit, `samples` cosine-weighted AO rays within ao_dist.
template <bool COUNT>
__device__ __forceinline__ PixelOut shade_pixel_ao(const SceneView &sc, const CameraView &cam, const MaterialView &mat,
                                                   int samples, float ao_dist, uint32_t seed, int x, int y,
                                                   uint32_t &status, FetchCount *fc)
{
    PixelOut out;
    out.secondary = 0;
    out.ao_made = 0;
    const RayState r = camera_ray(cam, x, y);
    HitRecord h;
    bool occ;
    status |= traverse<false, COUNT>(sc, r.o, r.d, FLT_MAX, h, occ, fc);
    out.hit = h.t < FLT_MAX;
    out.id = out.hit ? h.id - sc.tri_base : -1;
    out.c = cam.background;
    if (out.hit) {
        const uint32_t pix = (uint32_t)x + (uint32_t)y * (uint32_t)cam.xres;
        const SurfacePoint sp = surface_at(sc, r, h);
        const float3 start = offset_start(sp.dst, sp.geo);
        const AOBasis ob = ao_basis(sp.geo);
        int made = 0;
        for (int s = 0; s < samples; ++s) {
            const float3 d = ao_direction(ob, pix, (uint32_t)s, seed);
            HitRecord ah;
            bool blocked;
            status |= traverse<true, COUNT>(sc, start, d, ao_dist, ah, blocked, fc);
            if (!blocked) ++made;
        }
        const float3 kd = material_kd(mat, sp);
        const float frac = xdiv((float)made, (float)samples);
        out.c = xadd3(xmul3(kd, frac), mat.ka);
        out.secondary = (uint32_t)samples;
        out.ao_made = made;
    }
    return out;
}

// Shading state a lane keeps (in shared memory) while it traces the
// secondary rays of its pixel (lane-replacement kernels).
struct LaneShade {
    float3 kd, sn, start, c, vd, geo;
    int32_t id;
    int32_t made;          // AO: unoccluded rays; lights: blocked-light bits
};

__device__ __forceinline__ void store_rgb(uint8_t *rgb, size_t pix, float3 c)
{
    rgb[3 * pix] = clip8(c.x);
    rgb[3 * pix + 1] = clip8(c.y);
    rgb[3 * pix + 2] = clip8(c.z);
}

}  // namespace rtc
