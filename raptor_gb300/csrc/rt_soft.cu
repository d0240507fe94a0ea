// rt_soft.cu -- soft shadows as RAPTor renders them when it is built with
// SOFT_SHADOW = samples: every primary hit sends `samples` shadow rays to
// random points of each spherical (point or spot) or triangle-defined light
// and one to each directional light; a light's term is shaded with its
// first ray's direction and length and weighted by the fraction of rays that
// reach the light (ray::find_rays ray.cc:91-104, light::find_rays
// light.h:62-164, triangle::find_rays triangle.h:504-525,
// ray_trace_engine::ray_trace raytracer.cc:44-64).
//
// The random points come from the reference's own generator, one process-
// wide stream (common/common.cc:35-105) that the reference draws from in
// pixel order (x + y * xres) and, within a pixel, in light order: three
// numbers per ray of a spherical light, two per ray a triangle-defined
// light makes.  A pixel's position in that stream
// is therefore fixed by how many pixels before it hit something, so a frame
// is rendered in two passes: the camera rays first (hit records kept, one
// flag per pixel), an exclusive scan of the flags (each hit draws the same
// count), the frame's slice of the stream generated on the host and copied
// to the device, then the shading pass, every pixel reading its own slice.
// The cosine table the offsets go through (common/common.h:171-209) is
// built on the host the same way and kept on the device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include <cub/cub.cuh>

#include "rt_api_internal.cuh"
#include "rt_shade.cuh"

namespace rtc {

constexpr float kRefPi = 3.1415926535897932384626433f;   // common/common.cc:10
constexpr int kCosLutSize = 16384;                          // COS_LUT_SIZE, common/common.h:109-111

namespace {

// The reference's generator: a Mersenne twister seeded with 5489 whose
// refill updates words 0..622 only, tempered and scaled to [0, 1] in
// binary32.  pos counts the numbers produced since seeding.
struct RefRandom {
    uint32_t mt[624];
    int idx = 624;
    int64_t pos = 0;

    RefRandom() { reset(); }

    void reset()
    {
        mt[0] = 5489u;
        for (int i = 1; i < 624; ++i) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
        idx = 624;
        pos = 0;
    }

    void refill()
    {
        for (int i = 0; i < 227; ++i) {
            const uint32_t y = (0x80000000u & mt[i]) + (0x7FFFFFFFu & mt[i + 1]);
            mt[i] = mt[i + 397] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        for (int i = 227; i < 623; ++i) {
            const uint32_t y = (0x80000000u & mt[i]) + (0x7FFFFFFFu & mt[i + 1]);
            mt[i] = mt[i - 227] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        idx = 0;
    }

    float next()
    {
        if (idx >= 624) refill();
        uint32_t y = mt[idx++];
        ++pos;
        y ^= (y >> 11);
        y ^= ((y << 7) & 0x9d2c5680u);
        y ^= ((y << 15) & 0xefc60000u);
        y ^= (y >> 18);
        return (float)y * (1.0f / 4294967296.0f);
    }

    // Position the generator so that the next number is number p.
    void seek(int64_t p)
    {
        if (p < pos) reset();
        while (pos < p) {
            if (idx >= 624 && p - pos >= 624) {   // skip whole blocks without tempering
                refill();
                idx = 624;
                pos += 624;
                continue;
            }
            (void)next();
        }
    }
};

// Numbers [offset, offset + total) of the stream into out.  The state only
// changes at refills, so one pass walks the slice refill by refill
// (without tempering) and keeps a copy of the generator at the start of
// every chunk; host threads then temper their chunks in parallel.  The
// generator is left at offset + total.
void generate_slice(RefRandom &rng, int64_t offset, int64_t total, float *out)
{
    rng.seek(offset);
    constexpr int64_t kChunk = 624 * 2048;
    std::vector<RefRandom> starts;
    std::vector<int64_t> begins;
    for (int64_t b = 0; b < total; b += kChunk) {
        starts.push_back(rng);
        begins.push_back(b);
        rng.seek(offset + std::min(total, b + kChunk));
    }
    const int tasks = (int)starts.size();
    const int nthreads = std::max(1, std::min<int>(tasks, (int)std::thread::hardware_concurrency()));
    auto work = [&](int first) {
        for (int t = first; t < tasks; t += nthreads) {
            RefRandom g = starts[(size_t)t];
            const int64_t end = std::min(total, begins[(size_t)t] + kChunk);
            for (int64_t i = begins[(size_t)t]; i < end; ++i) out[i] = g.next();
        }
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < nthreads; ++k) pool.emplace_back(work, k);
    work(0);
    for (std::thread &th : pool) th.join();
}

// The rays light::find_rays makes for a triangle-defined light of ntris
// triangles asked for n (light.h:129-164): n / ntris per triangle, one more
// for every triangle the binary32 stride lands on.  cnt (ntris entries,
// nullable) receives the counts; returns their sum.
int32_t area_light_rays(int32_t ntris, int32_t n, int32_t *cnt)
{
    const int32_t ppt = n / ntris;
    const int32_t extra = n - ntris * ppt;
    const float stride = (float)ntris / (float)std::max(extra, 1);
    float at = 0.0f;
    int32_t made = 0;
    for (int32_t j = 0; j < ntris; ++j) {
        int32_t k = ppt;
        if (j == (int32_t)at) {
            ++k;
            at += stride;
        }
        if (cnt) cnt[j] = k;
        made += k;
    }
    return made;
}

}  // namespace

// Per-context state of the soft-shadow path.
struct SoftState {
    DevBuf lut;                  // the cosine table
    bool lut_ready = false;
    DevBuf hits;                 // int4 per pixel: the primary hit record
    DevBuf flags, prefix;        // int per pixel: hit flag, exclusive scan of the flags
    DevBuf scan_temp;
    DevBuf window;               // numbers [win_base, win_base + win_len) of the stream
    DevBuf area;                 // int4 per ray of a triangle-defined light: triangle, its rays, index
    int64_t win_base = -1, win_len = 0;
    RefRandom rng;
    float *staging = nullptr;    // pinned host copy of the slice being uploaded
    size_t staging_cap = 0;
};

void soft_release(rt_context *ctx)
{
    if (!ctx->soft) return;
    ctx->soft->lut.release();
    ctx->soft->hits.release();
    ctx->soft->flags.release();
    ctx->soft->prefix.release();
    ctx->soft->scan_temp.release();
    ctx->soft->window.release();
    ctx->soft->area.release();
    if (ctx->soft->staging) cudaFreeHost(ctx->soft->staging);
    delete ctx->soft;
    ctx->soft = nullptr;
}

namespace {

// static_cos::get_cos / get_sin (common/common.h:186-198): the index
// truncates toward zero and wraps modulo the table size (how the unsigned
// conversion of a negative angle behaves on the reference's x86-64 build).
__device__ __forceinline__ float lut_cos(const float *__restrict__ lut, float a)
{
    const float k = xmul(xdiv(1.0f, xmul(2.0f, kRefPi)), (float)kCosLutSize);
    const float v = xmul(k, a);
    long long e = 0;
    if (v > -9.2e18f && v < 9.2e18f) e = __float2ll_rz(v);
    return __ldg(lut + ((uint32_t)e & (uint32_t)(kCosLutSize - 1)));
}
__device__ __forceinline__ float lut_sin(const float *__restrict__ lut, float a)
{
    return lut_cos(lut, xsub(a, xdiv(kRefPi, 2.0f)));
}

// Shadow ray i of n to spherical light L: a random offset of the light's
// centre from rnd[0..2] (light.h:102-128), then ray::set_up(start,
// centre + offset) (ray.h:44-54).
__device__ __forceinline__ void soft_ray(const LightView &L, const float *__restrict__ lut, float3 start, int n,
                                         int i, const float *__restrict__ rnd, float3 &dir, float &len)
{
    const float a_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0xe) != 0) + 1));
    const float b_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0xc) != 0) + 1));
    const float r_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0x8) != 0) + 1));
    const int eighths = (i >> 2) & ~0x1;
    const float two_pi = xmul(2.0f, kRefPi);
    const float a_off = xmul(xmul(__ldg(rnd), xmul(a_scale, (float)(eighths + (i & 0x1)))), two_pi);
    const float b_off = xmul(xmul(__ldg(rnd + 1), xmul(b_scale, (float)(eighths + (i & 0x2)))), two_pi);
    const float r_off = xmul(xmul(__ldg(rnd + 2), xmul(r_scale, (float)(eighths + (i & 0x4)))), L.radius);
    const float sin_a = lut_sin(lut, a_off), cos_a = lut_cos(lut, a_off);
    const float sin_b = lut_sin(lut, b_off), cos_b = lut_cos(lut, b_off);
    const float3 off = make_float3(xmul(xmul(r_off, cos_a), sin_b), xmul(xmul(r_off, sin_a), sin_b), xmul(r_off, cos_b));
    const float3 dv = xsub3(xadd3(L.pos, off), start);
    len = xmag(dv);
    dir = xdiv3(dv, len);
}

// Shadow ray to triangle-defined light point e = (triangle, rays it makes,
// index of this one): barycentrics from rnd[0..1] (triangle.h:504-525),
// then ray::set_up(start, point).
__device__ __forceinline__ void area_ray(const float *__restrict__ verts, const int3 *__restrict__ idx, int4 e,
                                         float3 start, const float *__restrict__ rnd, float3 &dir, float &len)
{
    const int n = e.y, i = e.z;
    const float beta_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0xe) != 0) + 1));
    const float gamma_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0xc) != 0) + 1));
    const int eighths = (i >> 2) & ~0x1;
    const float beta = xmul(__ldg(rnd), xmul(beta_scale, (float)(eighths + (i & 0x1))));
    const float gamma = xmul(xmul(__ldg(rnd + 1), xmul(gamma_scale, (float)(eighths + (i & 0x2)))), xsub(1.0f, beta));
    const float alpha = xsub(1.0f, xadd(beta, gamma));
    const int3 t = idx[e.x];
    const float3 a = make_float3(__ldg(verts + 3 * t.x), __ldg(verts + 3 * t.x + 1), __ldg(verts + 3 * t.x + 2));
    const float3 b = make_float3(__ldg(verts + 3 * t.y), __ldg(verts + 3 * t.y + 1), __ldg(verts + 3 * t.y + 2));
    const float3 c = make_float3(__ldg(verts + 3 * t.z), __ldg(verts + 3 * t.z + 1), __ldg(verts + 3 * t.z + 2));
    const float3 p = xadd3(xadd3(xmul3(a, alpha), xmul3(b, beta)), xmul3(c, gamma));
    const float3 dv = xsub3(p, start);
    len = xmag(dv);
    dir = xdiv3(dv, len);
}

__device__ __forceinline__ bool soft_light(const LightView &L, int samples)
{
    return samples > 1 && L.kind != RT_LIGHT_DIRECTIONAL;
}

// Per light: first entry of its rays in the ray table and the rays it
// makes (0: not triangle-defined); numbers a hit draws for it.
struct AreaSet {
    int32_t first[RT_MAX_LIGHTS];
    int32_t made[RT_MAX_LIGHTS];
    int32_t draws[RT_MAX_LIGHTS];
};

// Pass 1: the camera ray of every pixel; hit record and hit flag.
__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_soft_primary(SceneView sc, CameraView cam,
                                                                                      int4 *__restrict__ hits,
                                                                                      int32_t *__restrict__ flags,
                                                                                      Counters *ctr)
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
        if (live) {
            const RayState r = camera_ray(cam, x, y);
            HitRecord h;
            bool occ;
            status |= traverse<false>(sc, r.o, r.d, FLT_MAX, h, occ);
            hit = h.t < FLT_MAX;
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            hits[pix] = make_int4(h.id, __float_as_int(h.t), __float_as_int(h.u), __float_as_int(h.v));
            flags[pix] = hit ? 1 : 0;
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, hit);
    }
    if (status) atomicOr(&ctr->status, status);
}

// Pass 2: shading.  rnd holds the frame's numbers (rnd[0] = the frame's
// first), nrnd of them; a hit pixel's first is prefix[pix] * per_hit.
__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_soft_shade(
    SceneView sc, CameraView cam, LightSet lights, MaterialTable table, AreaSet areas, const int4 *__restrict__ area,
    const float *__restrict__ verts, int32_t samples, int32_t per_hit, const float *__restrict__ rnd, int64_t nrnd,
    const float *__restrict__ lut, const int4 *__restrict__ hits, const int32_t *__restrict__ prefix,
    uint8_t *__restrict__ rgb, float *__restrict__ fimg, Counters *ctr)
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
        uint32_t nsec = 0;
        if (live) {
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            const int4 hr = hits[pix];
            float3 c = cam.background;
            if (__int_as_float(hr.y) < FLT_MAX) {
                HitRecord h;
                h.id = hr.x;
                h.t = __int_as_float(hr.y);
                h.u = __int_as_float(hr.z);
                h.v = __int_as_float(hr.w);
                const RayState r = camera_ray(cam, x, y);
                int32_t mi = 0;
                if (sc.mat) {
                    mi = __ldg(&sc.mat[h.id - sc.tri_base]);
                    if (mi < 0 || mi >= table.n) { status |= kStatusBadIndex; mi = 0; }
                }
                const MaterialView &mat = table.m[mi];
                const SurfacePoint sp = surface_at(sc, r, h);
                const float3 start = offset_start(sp.dst, sp.geo);
                const float3 kd = material_kd(mat, sp);
                int64_t draw = (int64_t)prefix[pix] * per_hit;
                c = make_float3(0.f, 0.f, 0.f);
                for (int l = 0; l < lights.n; ++l) {
                    const LightView &L = lights.l[l];
                    float3 ldir;
                    float len;
                    int n = 1, made = 0;
                    if (soft_light(L, samples)) {
                        n = samples;
                        if (draw + (int64_t)areas.draws[l] > nrnd) {   // never expected: the host sized the slice
                            status |= kStatusBadIndex;
                            break;
                        }
                        const bool tri_light = areas.made[l] > 0;
                        for (int i = 0; i < n; ++i) {
                            float3 di;
                            float li;
                            if (tri_light)
                                area_ray(verts, sc.idx, __ldg(area + areas.first[l] + i), start, rnd + draw + 2 * i,
                                         di, li);
                            else
                                soft_ray(L, lut, start, n, i, rnd + draw + 3 * i, di, li);
                            if (i == 0) { ldir = di; len = li; }
                            HitRecord sh;
                            bool blocked;
                            status |= traverse<true>(sc, start, di, li, sh, blocked);
                            if (!blocked) ++made;
                        }
                        draw += areas.draws[l];
                    } else {
                        shadow_ray(L, start, ldir, len);
                        HitRecord sh;
                        bool blocked;
                        status |= traverse<true>(sc, start, ldir, len, sh, blocked);
                        made = blocked ? 0 : 1;
                    }
                    nsec += (uint32_t)n;
                    // made_it / nr_pending_shadows, both floats (raytracer.cc:46-61)
                    phong_add<true>(L, mat, kd, sp.sn, r.d, ldir, len, xdiv((float)made, (float)n), c);
                }
                c = xadd3(c, mat.ka);
            }
            if (rgb) store_rgb(rgb, pix, c);
            if (fimg) {
                fimg[3 * pix] = c.x;
                fimg[3 * pix + 1] = c.y;
                fimg[3 * pix + 2] = c.z;
            }
        }
        warp_add(&ctr->secondary, nsec);
    }
    if (status) atomicOr(&ctr->status, status);
}

}  // namespace
}  // namespace rtc

using namespace rtc;

namespace {

rt_status sfail(rt_status c, const char *m) { return set_error(c, m); }

#define RT_CUDA_S(call, what)                                  \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return set_cuda_error(_e, what); \
    } while (0)

struct SGuard {
    int prev = -1;
    explicit SGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~SGuard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

int soft_blocks_per_sm()
{
    static const int per_sm = [] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_soft_shade, kTraceThreads, 0) != cudaSuccess || b < 1) {
            cudaGetLastError();
            b = 4;
        }
        return b;
    }();
    return per_sm;
}

}  // namespace

extern "C" rt_status rt_render_soft_shadows(rt_scene *s, const rt_camera *camera, const rt_light *lights,
                                            int32_t nlights, const rt_light_shape *shapes,
                                            const rt_material *materials, int32_t nmaterials, int32_t samples,
                                            int64_t stream_offset, uint8_t *rgb_out, float *rgb_f32,
                                            int64_t *stream_end, rt_render_stats *stats)
{
    if (!s || !camera || !materials || (!rgb_out && !rgb_f32))
        return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: NULL argument");
    if (camera->xres <= 0 || camera->yres <= 0 || (int64_t)camera->xres * camera->yres > (int64_t)1 << 28)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: camera resolution out of range");
    if (nlights < 0 || nlights > RT_MAX_LIGHTS || (nlights > 0 && !lights))
        return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: light count out of range");
    if (nmaterials < 1 || nmaterials > RT_MAX_MATERIALS)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: material count must be 1..RT_MAX_MATERIALS");
    if (samples < 1 || samples > RT_MAX_SOFT_SAMPLES)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: samples must be 1..RT_MAX_SOFT_SAMPLES");
    if (stream_offset < 0) return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: negative stream offset");
    for (int32_t i = 0; i < nmaterials; ++i)
        if (materials[i].rf != 0.0f || materials[i].tran != 0.0f)
            return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: mirror and refracting materials are not offered");
    for (int32_t i = 0; i < nlights && shapes; ++i) {
        const rt_light_shape &sh = shapes[i];
        if (!(sh.radius >= 0.0f && sh.radius < 3.0e38f))
            return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: light radius must be finite and >= 0");
        if (sh.ntris < 0 || (sh.ntris > 0 && !sh.tris))
            return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: bad triangle list of a light");
        if (sh.ntris > 0 && (sh.radius != 0.0f || lights[i].kind == RT_LIGHT_DIRECTIONAL))
            return sfail(RT_ERR_INVALID_ARG,
                         "rt_render_soft_shadows: a triangle-defined light is a point or spot light of radius 0");
        for (int32_t j = 0; j < sh.ntris; ++j)
            if (sh.tris[j] < 0 || sh.tris[j] >= s->ntris)
                return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: light triangle index out of range");
    }
    if (!s->built) return sfail(RT_ERR_NOT_BUILT, "rt_render_soft_shadows: hierarchy not built");
    if (s->mat_max >= nmaterials)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: the scene's material indices exceed the table");
    rt_context *ctx = s->ctx;
    SGuard g(ctx->device);
    if (!ctx->soft) {
        ctx->soft = new (std::nothrow) SoftState();
        if (!ctx->soft) return sfail(RT_ERR_OUT_OF_MEMORY, "rt_render_soft_shadows: state allocation");
    }
    SoftState &S = *ctx->soft;
    cudaStream_t st = ctx->stream;
    if (!S.lut_ready) {
        // static_cos (common/common.h:174-181): angle rounded to binary32,
        // cosine in double, rounded to binary32
        std::vector<float> lut(kCosLutSize);
        for (int i = 0; i < kCosLutSize; ++i)
            lut[i] = (float)std::cos((double)((((float)i * 2.0f) * kRefPi) / (float)kCosLutSize));
        RT_CUDA_S(S.lut.reserve(kCosLutSize * sizeof(float)), "cosine table allocation");
        RT_CUDA_S(cudaMemcpy(S.lut.ptr, lut.data(), kCosLutSize * sizeof(float), cudaMemcpyHostToDevice),
                  "cosine table copy");
        S.lut_ready = true;
    }
    const size_t npix = (size_t)camera->xres * (size_t)camera->yres;
    RT_CUDA_S(S.hits.reserve(npix * sizeof(int4)), "hit record allocation");
    RT_CUDA_S(S.flags.reserve(npix * sizeof(int32_t)), "hit flag allocation");
    RT_CUDA_S(S.prefix.reserve(npix * sizeof(int32_t)), "prefix allocation");
    size_t scan_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (const int32_t *)S.flags.ptr, (int32_t *)S.prefix.ptr,
                                  (int)npix, st);
    RT_CUDA_S(S.scan_temp.reserve(scan_bytes), "scan scratch allocation");
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = 0;
    AreaSet as = {};
    std::vector<int4> area_rays;
    int32_t per_hit = 0;
    for (int i = 0; i < nlights; ++i) {
        ls.l[i] = make_light_view(lights[i]);
        ls.l[i].radius = shapes ? shapes[i].radius : 0.0f;
        if (!(samples > 1 && ls.l[i].kind != RT_LIGHT_DIRECTIONAL)) continue;
        if (shapes && shapes[i].ntris > 0) {
            // the light's rays in the order find_rays makes them; the first
            // `samples` are traced, every one made draws two numbers
            const int32_t nt = shapes[i].ntris;
            std::vector<int32_t> cnt((size_t)nt);
            const int32_t made = area_light_rays(nt, samples, cnt.data());
            if (made < samples)
                return sfail(RT_ERR_INVALID_ARG,
                             "rt_render_soft_shadows: a triangle-defined light makes fewer rays than samples");
            as.first[i] = (int32_t)area_rays.size();
            as.made[i] = made;
            as.draws[i] = 2 * made;
            for (int32_t j = 0; j < nt; ++j)
                for (int32_t k = 0; k < cnt[(size_t)j]; ++k) area_rays.push_back(make_int4(shapes[i].tris[j], cnt[(size_t)j], k, 0));
        } else {
            as.draws[i] = 3 * samples;
        }
        per_hit += as.draws[i];
    }
    if (!area_rays.empty()) {
        RT_CUDA_S(S.area.reserve(area_rays.size() * sizeof(int4)), "light ray table allocation");
        RT_CUDA_S(cudaMemcpyAsync(S.area.ptr, area_rays.data(), area_rays.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                  st),
                  "light ray table copy");
    }
    MaterialTable mt;
    mt.n = nmaterials;
    for (int i = 0; i < nmaterials; ++i) mt.m[i] = make_material_view(materials[i]);
    const SceneView sv = scene_view(s);
    const CameraView cv = make_camera_view(*camera);
    const int grid = soft_blocks_per_sm() * ctx->sm_count;

    RT_CUDA_S(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), st), "counter clear");
    RT_CUDA_S(cudaEventRecord(ctx->ev0, st), "event record");
    k_soft_primary<<<grid, kTraceThreads, 0, st>>>(sv, cv, (int4 *)S.hits.ptr, (int32_t *)S.flags.ptr, ctx->d_counters);
    RT_CUDA_S(cudaGetLastError(), "primary launch");
    cub::DeviceScan::ExclusiveSum(S.scan_temp.ptr, scan_bytes, (const int32_t *)S.flags.ptr, (int32_t *)S.prefix.ptr,
                                  (int)npix, st);
    RT_CUDA_S(cudaGetLastError(), "scan launch");
    // the frame's count of numbers: per_hit for every hit pixel
    int32_t *h = ctx->h_scratch;
    RT_CUDA_S(cudaMemcpyAsync(h, (const int32_t *)S.prefix.ptr + (npix - 1), sizeof(int32_t), cudaMemcpyDeviceToHost, st),
              "prefix read");
    RT_CUDA_S(cudaMemcpyAsync(h + 1, (const int32_t *)S.flags.ptr + (npix - 1), sizeof(int32_t),
                              cudaMemcpyDeviceToHost, st),
              "flag read");
    RT_CUDA_S(cudaStreamSynchronize(st), "synchronize");
    const int64_t nhits = (int64_t)h[0] + h[1];
    const int64_t total = nhits * per_hit;
    // the frame's slice of the reference's stream, kept on the device while
    // later frames fall inside it
    if (total > 0 && !(S.win_base >= 0 && stream_offset >= S.win_base &&
                       stream_offset + total <= S.win_base + S.win_len)) {
        if (S.staging_cap < (size_t)total) {
            if (S.staging) cudaFreeHost(S.staging);
            S.staging = nullptr;
            S.staging_cap = 0;
            const size_t cap = (size_t)total + (size_t)total / 4;
            RT_CUDA_S(cudaMallocHost(&S.staging, cap * sizeof(float)), "pinned stream staging");
            S.staging_cap = cap;
        }
        generate_slice(S.rng, stream_offset, total, S.staging);
        RT_CUDA_S(S.window.reserve((size_t)total * sizeof(float)), "stream allocation");
        RT_CUDA_S(cudaMemcpyAsync(S.window.ptr, S.staging, (size_t)total * sizeof(float), cudaMemcpyHostToDevice, st),
                  "stream copy");
        S.win_base = stream_offset;
        S.win_len = total;
    }
    const float *rnd = total > 0 ? (const float *)S.window.ptr + (stream_offset - S.win_base) : nullptr;

    // outputs: device pointers as given, host ones staged
    const bool rgb_host = rgb_out && !is_device_ptr(rgb_out);
    const bool f_host = rgb_f32 && !is_device_ptr(rgb_f32);
    uint8_t *d_rgb = rgb_out;
    float *d_f = rgb_f32;
    if (rgb_host) {
        RT_CUDA_S(ctx->stage_a.reserve(npix * 3), "staging allocation");
        d_rgb = (uint8_t *)ctx->stage_a.ptr;
    }
    if (f_host) {
        RT_CUDA_S(ctx->fimg.reserve(npix * 3 * sizeof(float)), "float frame allocation");
        d_f = (float *)ctx->fimg.ptr;
    }
    RT_CUDA_S(cudaMemsetAsync(&ctx->d_counters->work, 0, sizeof(int), st), "work counter clear");
    k_soft_shade<<<grid, kTraceThreads, 0, st>>>(sv, cv, ls, mt, as, (const int4 *)S.area.ptr, s->d_verts, samples,
                                                 per_hit, rnd, total, (const float *)S.lut.ptr,
                                                 (const int4 *)S.hits.ptr, (const int32_t *)S.prefix.ptr, d_rgb, d_f,
                                                 ctx->d_counters);
    RT_CUDA_S(cudaGetLastError(), "shade launch");
    RT_CUDA_S(cudaEventRecord(ctx->ev1, st), "event record");
    if (rgb_host) RT_CUDA_S(cudaMemcpyAsync(rgb_out, d_rgb, npix * 3, cudaMemcpyDeviceToHost, st), "rgb copy");
    if (f_host)
        RT_CUDA_S(cudaMemcpyAsync(rgb_f32, d_f, npix * 3 * sizeof(float), cudaMemcpyDeviceToHost, st), "image copy");
    Counters c;
    RT_CUDA_S(cudaMemcpyAsync(&c, ctx->d_counters, sizeof(Counters), cudaMemcpyDeviceToHost, st), "counter read");
    RT_CUDA_S(cudaStreamSynchronize(st), "synchronize");
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
    if (stream_end) *stream_end = stream_offset + total;
    return status_to_error(c.status);
}
