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
// (ray_trace_engine::ray_trace, raytracer.cc:20-87).  TABLE: the hit
// triangle's material from `table` (per-triangle indices in sc.mat), else
// `mat0` for every triangle.
template <bool COUNT, bool TABLE = false, int STACK = kStackSize>
__device__ __forceinline__ PixelOut shade_pixel_lights(const SceneView &sc, const CameraView &cam, const LightView *lights,
                                                       int nl, const MaterialView &mat0, int x, int y,
                                                       uint32_t &status, FetchCount *fc, bool fast_pow,
                                                       const MaterialTable *table = nullptr)
{
    PixelOut out;
    out.secondary = 0;
    out.ao_made = 0;
    const RayState r = camera_ray(cam, x, y);
    HitRecord h;
    bool occ;
    status |= traverse<false, COUNT, STACK>(sc, r.o, r.d, FLT_MAX, h, occ, fc);
    out.hit = h.t < FLT_MAX;
    out.id = out.hit ? h.id - sc.tri_base : -1;
    out.c = cam.background;
    if (out.hit) {
        int32_t mi = 0;
        if (TABLE && sc.mat) {
            mi = __ldg(&sc.mat[out.id]);
            if (mi < 0 || mi >= table->n) { status |= kStatusBadIndex; mi = 0; }
        }
        const MaterialView &mat = TABLE ? table->m[mi] : mat0;
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
            status |= traverse<true, COUNT, STACK>(sc, start, ldir, len, sh, blocked, fc);
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

// One pending ray of a pixel's ray tree and, once it has hit, what its
// children need: the hit point and geometric normal (start points), the
// shading normal, the incoming direction, the material, and the colour
// accumulated so far.
struct TreeFrame {
    float3 o_or_dst;   // stage 0: ray origin; later: refined hit point
    float3 d;          // ray direction
    float3 sn, geo;
    float3 c;
    float magn;
    int32_t mat;
    int32_t stage;     // 0 trace, 1 reflection next, 2 refraction next, 3 done
    int32_t out_in;    // the ray entered the front face (hit_t::out_in)
};

// A pixel's ray tree (ray_trace_engine::ray_trace, raytracer.cc:20-87, as a
// post-order walk with an explicit stack): at every hit the coloured Phong
// of its triangle's material with the exact specular power; then the
// mirror ray (ray::reflect, ray.cc:118-135: power magn * rf, traced while it
// exceeds 0.1 compared in double) and the refracted ray (ray::refract,
// ray.cc:198-281: power magn * tran, ri inverted for a ray entering the
// front face, none beyond the critical angle, start point pushed into the
// surface), each child's colour added to its parent's times rf, then tran
// (combind_secondary_rays, coloured_mapper_shader.cc:117-130).  A ray that
// misses is the background.  `frames` holds RT_MAX_BOUNCES + 1 entries.
template <bool COUNT>
__device__ __forceinline__ PixelOut shade_pixel_tree(const SceneView &sc, const CameraView &cam, const LightView *lights,
                                                     int nl, const MaterialTable &mt, int x, int y, TreeFrame *frames,
                                                     uint32_t &status, FetchCount *fc)
{
    PixelOut out;
    out.secondary = 0;
    out.ao_made = 0;
    out.hit = false;
    out.id = -1;
    out.c = cam.background;
    const RayState cr = camera_ray(cam, x, y);
    int sp = 0;
    frames[0].o_or_dst = cr.o;
    frames[0].d = cr.d;
    frames[0].magn = 1.0f;
    frames[0].stage = 0;
    sp = 1;
    for (int guard = 0; sp > 0 && guard < 4 * RT_MAX_TREE_RAYS; ++guard) {
        TreeFrame &F = frames[sp - 1];
        if (F.stage == 0) {
            HitRecord h;
            bool occ;
            status |= traverse<false, COUNT>(sc, F.o_or_dst, F.d, FLT_MAX, h, occ, fc);
            if (sp > 1) ++out.secondary;
            if (!(h.t < FLT_MAX)) {
                // background; deliver to the parent below
                F.c = cam.background;
                F.stage = 3;
            } else {
                const int32_t id = h.id - sc.tri_base;
                if (sp == 1) {
                    out.hit = true;
                    out.id = id;
                }
                int32_t mi = sc.mat ? __ldg(&sc.mat[id]) : 0;
                if (mi < 0 || mi >= mt.n) { status |= kStatusBadIndex; mi = 0; }
                const MaterialView &m = mt.m[mi];
                RayState r;
                r.o = F.o_or_dst;
                r.d = F.d;
                const SurfacePoint spt = surface_at(sc, r, h);
                const float3 start = offset_start(spt.dst, spt.geo);
                const float3 kd = material_kd(m, spt);
                float3 c = make_float3(0.f, 0.f, 0.f);
                for (int l = 0; l < nl; ++l) {
                    float3 ldir;
                    float len;
                    shadow_ray(lights[l], start, ldir, len);
                    HitRecord shh;
                    bool blocked;
                    status |= traverse<true, COUNT>(sc, start, ldir, len, shh, blocked, fc);
                    ++out.secondary;
                    phong_add<true>(lights[l], m, kd, spt.sn, F.d, ldir, len, blocked ? 0.0f : 1.0f, c);
                }
                F.c = xadd3(c, m.ka);
                F.o_or_dst = spt.dst;
                F.sn = spt.sn;
                F.geo = spt.geo;
                F.mat = mi;
                F.out_in = spt.out_in ? 1 : 0;
                F.stage = 1;
            }
        }
        if (F.stage == 1) {
            F.stage = 2;
            const MaterialView &m = mt.m[F.mat];
            const float power = xmul(F.magn, m.rf);
            if ((double)power > 0.1) {
                if (sp > RT_MAX_BOUNCES) { status |= kStatusStepLimit; }
                else {
                    TreeFrame &C = frames[sp];
                    const float rdn = xmul(2.0f, xdot(F.d, F.sn));
                    C.o_or_dst = offset_start(F.o_or_dst, F.geo);
                    C.d = xsub3(F.d, xmul3(F.sn, rdn));
                    C.magn = power;
                    C.stage = 0;
                    ++sp;
                    continue;
                }
            }
        }
        if (F.stage == 2) {
            F.stage = 3;
            const MaterialView &m = mt.m[F.mat];
            const float power = xmul(F.magn, m.tran);
            if ((double)power > 0.1) {
                float ri = m.ri;
                const float rdn = -xdot(F.d, F.sn);
                if (F.out_in) ri = xdiv(1.0f, ri);
                const float cos_t2 = xsub(1.0f, xmul(xmul(ri, ri), xsub(1.0f, xmul(rdn, rdn))));
                if (!(cos_t2 < 0.0f)) {
                    if (sp > RT_MAX_BOUNCES) { status |= kStatusStepLimit; }
                    else {
                        const float off = xsub(xmul(ri, rdn), __fsqrt_rn(cos_t2));
                        TreeFrame &C = frames[sp];
                        C.o_or_dst = offset_start_in(F.o_or_dst, F.geo);
                        C.d = xadd3(xmul3(F.d, ri), xmul3(F.sn, off));
                        C.magn = power;
                        C.stage = 0;
                        ++sp;
                        continue;
                    }
                }
            }
        }
        // stage 3: the frame's colour is complete; deliver it to its parent
        const float3 col = F.c;
        --sp;
        if (sp == 0) {
            out.c = col;
        } else {
            TreeFrame &P = frames[sp - 1];
            const MaterialView &pm = mt.m[P.mat];
            // P.stage is 2 after its mirror child, 3 after its refracted child
            const float w = (P.stage == 2) ? pm.rf : pm.tran;
            P.c = xadd3(P.c, xmul3(xadd3(make_float3(0.f, 0.f, 0.f), col), w));
        }
    }
    if (sp > 0) status |= kStatusStepLimit;
    return out;
}

// Primary ray, closest hit, `samples` cosine-weighted AO rays within ao_dist.
template <bool COUNT, int STACK = kStackSize>
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
    status |= traverse<false, COUNT, STACK>(sc, r.o, r.d, FLT_MAX, h, occ, fc);
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
            status |= traverse<true, COUNT, STACK>(sc, start, d, ao_dist, ah, blocked, fc);
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
