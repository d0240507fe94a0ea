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
    // worker k tempers chunks k, k + nthreads, ...; the workers whose thread
    // could not be started run here, one after another, once the rest are done
    std::vector<std::thread> pool;
    int started = 1;
    try {
        for (int k = 1; k < nthreads; ++k) {
            pool.emplace_back(work, k);
            ++started;
        }
    } catch (...) {
    }
    work(0);
    for (std::thread &th : pool) th.join();
    for (int k = started; k < nthreads; ++k) work(k);
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
    DevBuf counts, prefix64;     // int64 per pixel: numbers a distributed pixel draws, their exclusive scan
    DevBuf scan64_temp;
    // distributed frames on per-pixel streams: each pixel's camera-ray node
    // (colour, material; first item, set sizes), the items (its sets' rays),
    // their subtrees' colours, the item count
    DevBuf root_c, root_sets, items, item_c, nitems;
    int64_t item_cap = 0;
    int64_t win_base = -1, win_len = 0;
    // Host side of the stream: staging holds numbers [stage_base, stage_base
    // + stage_len) and rng stands at their end.  After each upload a thread
    // reads ahead: it generates the numbers that follow the frame's slice
    // (where the next frame starts, drawing about as many) while the GPU
    // renders; the next window joins it first.
    RefRandom rng;
    float *staging = nullptr;    // pinned
    size_t staging_cap = 0;
    int64_t stage_base = -1, stage_len = 0;
    std::thread ahead;
    cudaEvent_t copied = nullptr;   // the last upload out of staging
    int device = 0;
};

// Waits for a read-ahead in flight.
void join_ahead(SoftState &S)
{
    if (S.ahead.joinable()) S.ahead.join();
}

void soft_release(rt_context *ctx)
{
    if (!ctx->soft) return;
    join_ahead(*ctx->soft);
    if (ctx->soft->copied) cudaEventDestroy(ctx->soft->copied);
    ctx->soft->lut.release();
    ctx->soft->hits.release();
    ctx->soft->flags.release();
    ctx->soft->prefix.release();
    ctx->soft->scan_temp.release();
    ctx->soft->window.release();
    ctx->soft->area.release();
    ctx->soft->counts.release();
    ctx->soft->prefix64.release();
    ctx->soft->scan64_temp.release();
    ctx->soft->root_c.release();
    ctx->soft->root_sets.release();
    ctx->soft->items.release();
    ctx->soft->item_c.release();
    ctx->soft->nitems.release();
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
// centre from the numbers u0, u1, u2 (light.h:102-128), then
// ray::set_up(start, centre + offset) (ray.h:44-54).
__device__ __forceinline__ void soft_ray(const LightView &L, const float *__restrict__ lut, float3 start, int n,
                                         int i, float u0, float u1, float u2, float3 &dir, float &len)
{
    const float a_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0xe) != 0) + 1));
    const float b_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0xc) != 0) + 1));
    const float r_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0x8) != 0) + 1));
    const int eighths = (i >> 2) & ~0x1;
    const float two_pi = xmul(2.0f, kRefPi);
    const float a_off = xmul(xmul(u0, xmul(a_scale, (float)(eighths + (i & 0x1)))), two_pi);
    const float b_off = xmul(xmul(u1, xmul(b_scale, (float)(eighths + (i & 0x2)))), two_pi);
    const float r_off = xmul(xmul(u2, xmul(r_scale, (float)(eighths + (i & 0x4)))), L.radius);
    const float sin_a = lut_sin(lut, a_off), cos_a = lut_cos(lut, a_off);
    const float sin_b = lut_sin(lut, b_off), cos_b = lut_cos(lut, b_off);
    const float3 off = make_float3(xmul(xmul(r_off, cos_a), sin_b), xmul(xmul(r_off, sin_a), sin_b), xmul(r_off, cos_b));
    const float3 dv = xsub3(xadd3(L.pos, off), start);
    len = xmag(dv);
    dir = xdiv3(dv, len);
}

// Shadow ray to triangle-defined light point e = (triangle, rays it makes,
// index of this one): barycentrics from the numbers u0, u1
// (triangle.h:504-525), then ray::set_up(start, point).
__device__ __forceinline__ void area_ray(const float *__restrict__ verts, const int3 *__restrict__ idx, int4 e,
                                         float3 start, float u0, float u1, float3 &dir, float &len)
{
    const int n = e.y, i = e.z;
    const float beta_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0xe) != 0) + 1));
    const float gamma_scale = xdiv(1.0f, (float)((n >> 4) + ((n & 0xc) != 0) + 1));
    const int eighths = (i >> 2) & ~0x1;
    const float beta = xmul(u0, xmul(beta_scale, (float)(eighths + (i & 0x1))));
    const float gamma = xmul(xmul(u1, xmul(gamma_scale, (float)(eighths + (i & 0x2)))), xsub(1.0f, beta));
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
                            if (tri_light) {
                                const float *u = rnd + draw + 2 * i;
                                area_ray(verts, sc.idx, __ldg(area + areas.first[l] + i), start, __ldg(u),
                                         __ldg(u + 1), di, li);
                            } else {
                                const float *u = rnd + draw + 3 * i;
                                soft_ray(L, lut, start, n, i, __ldg(u), __ldg(u + 1), __ldg(u + 2), di, li);
                            }
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

// ------------------------------------------------ distributed ray tracing

// Frames of a pixel's ray tree: one per level below the camera ray.
constexpr int kDistDepth = RT_MAX_BOUNCES + 1;
// Componant levels with their own counts: componant 4^k for k < 4; with
// at most 64 samples every count max(samples / 4^k, 1) is 1 from k = 3 on.
constexpr int kDistLevels = 4;

// Per light and componant level: the first entry of the light's rays in
// the ray table and the rays it makes (0: not triangle-defined), and the
// numbers one hit draws for it.
struct DistLights {
    int32_t first[RT_MAX_LIGHTS][kDistLevels];
    int32_t made[RT_MAX_LIGHTS][kDistLevels];
    int32_t draws[RT_MAX_LIGHTS][kDistLevels];
};

struct DistParams {
    int32_t soft, diffuse;
    int32_t pixel_stream;        // 1: per-pixel Philox streams; 0: the frame's slice of the reference's
    uint32_t key0, key1;
    int32_t max_steps;           // frame visits per pixel (bounded by the tree's worst case)
    float rfd[RT_MAX_MATERIALS];
    float td[RT_MAX_MATERIALS];
};

// Tree nodes of a pixel's per-pixel streams: the camera ray is kTreeRoot;
// ray `index` of a node's reflection (set 0) or refraction (set 1) set is
// SplitMix64 (Steele, Lea and Flood 2014) of node + (64 set + index + 1) *
// 0x9E3779B97F4A7C15.
constexpr uint64_t kTreeRoot = 0x6A09E667F3BCC909ull;
__device__ __forceinline__ uint64_t tree_child(uint64_t parent, int set, int index)
{
    uint64_t z = parent + (uint64_t)(set * 64 + index + 1) * 0x9E3779B97F4A7C15ull + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// A pixel's random numbers: number k that tree node `node` draws from the
// pixel's Philox streams (counter (pixel, node low, node high, k / 4)), or
// number base + k of the frame's slice of the reference's stream (k the
// pixel's running index; node unused).
struct DistStream {
    const float *win;
    int64_t base, nwin;
    uint32_t pixel, key0, key1;
    bool pixel_mode;
    uint32_t blk;                // last Philox block computed, and its node
    uint64_t bnode;
    uint4 w;

    __device__ __forceinline__ float at(uint64_t node, uint32_t k, uint32_t &status)
    {
        if (pixel_mode) {
            if ((k >> 2) != blk || node != bnode) {
                blk = k >> 2;
                bnode = node;
                w = philox4x32(make_uint4(pixel, (uint32_t)node, (uint32_t)(node >> 32), blk), key0, key1);
            }
            const uint32_t u = (k & 3u) == 0u ? w.x : (k & 3u) == 1u ? w.y : (k & 3u) == 2u ? w.z : w.w;
            return xmul(__uint2float_rn(u), 2.3283064365386963e-10f);
        }
        const int64_t i = base + (int64_t)k;
        if (i < 0 || i >= nwin) {   // never expected: the host sized the slice
            status |= kStatusBadIndex;
            return 0.0f;
        }
        return __ldg(win + i);
    }
};

// One ray of a diffuse set about direction ref (ray::reflect
// ray.cc:137-182, ray::refract ray.cc:236-280): ref + perpen * r cos a +
// cross * r sin a, with perpen = (ref.z, ref.y, -ref.x), cross = ref x
// perpen, r = spread * u0, a = 2 pi * u1 through the cosine table; the
// direction is not normalised.
__device__ __forceinline__ float3 spread_dir(float3 ref, float spread, float u0, float u1, const float *__restrict__ lut)
{
    const float3 perpen = make_float3(ref.z, ref.y, -ref.x);
    const float3 cr = xcross(ref, perpen);
    const float r_off = xmul(u0, spread);
    const float a_off = xmul(u1, xmul(2.0f, kRefPi));
    const float x_off = xmul(r_off, lut_cos(lut, a_off));
    const float y_off = xmul(r_off, lut_sin(lut, a_off));
    return xadd3(xadd3(ref, xmul3(perpen, x_off)), xmul3(cr, y_off));
}

struct DistFrame {
    float3 o;            // the ray's origin; after its hit, the refined hit point
    float3 d;            // its direction
    float3 sn, geo;      // shading and geometric normal at the hit
    float3 c;            // its colour: the lights and ka, then the sets' means
    float3 sum;          // colours of the current set's rays so far
    float magn;          // power
    int32_t level;       // componant 4^level
    uint64_t node;       // its tree node (per-pixel streams)
    int32_t mat;
    int32_t stage;
    int32_t out_in;
    int32_t nrefl, nrefr, child;
    uint32_t refl_at, refr_at;   // the pixel's number index of each set's first number
};

enum : int32_t { kDistTrace = 0, kDistRefl = 1, kDistRefr = 2, kDistDone = 3, kDistLights = 4 };

__device__ __forceinline__ int dist_count(int32_t samples, int32_t level)
{
    return max(samples >> (2 * min(level, kDistLevels - 1)), 1);
}

// Child ray i of frame f's reflection (set 0: ray::reflect ray.cc:118-182,
// power magn * rf) or refraction (set 1: ray::refract ray.cc:198-281, power
// magn * tran, ri inverted for a ray entering the front face, start point
// pushed into the surface) set, its direction spread by the set's numbers
// when the material spreads it.
__device__ __forceinline__ void spawn_child(const DistFrame &f, const MaterialView &m, const DistParams &dp, int set,
                                            int i, const float *__restrict__ lut, DistStream &S, uint32_t &status,
                                            DistFrame &C)
{
    if (set == 0) {
        const bool spread = dp.diffuse > 0 && dp.rfd[f.mat] != 0.0f;
        const float rdn = xmul(2.0f, xdot(f.d, f.sn));
        const float3 ref = xsub3(f.d, xmul3(f.sn, rdn));
        if (spread) {
            const uint32_t at = f.refl_at + 2u * (uint32_t)i;
            C.d = spread_dir(ref, dp.rfd[f.mat], S.at(f.node, at, status), S.at(f.node, at + 1, status), lut);
        } else {
            C.d = ref;
        }
        C.o = offset_start(f.o, f.geo);
        C.magn = xmul(f.magn, m.rf);
        C.level = f.level + (spread ? 1 : 0);
    } else {
        const bool spread = dp.diffuse > 0 && dp.td[f.mat] != 0.0f;
        float ri = m.ri;
        const float rdn = -xdot(f.d, f.sn);
        if (f.out_in) ri = xdiv(1.0f, ri);
        const float cos_t2 = xsub(1.0f, xmul(xmul(ri, ri), xsub(1.0f, xmul(rdn, rdn))));
        const float off = xsub(xmul(ri, rdn), __fsqrt_rn(cos_t2));
        const float3 ref = xadd3(xmul3(f.d, ri), xmul3(f.sn, off));
        if (spread) {
            const uint32_t at = f.refr_at + 2u * (uint32_t)i;
            C.d = spread_dir(ref, dp.td[f.mat], S.at(f.node, at, status), S.at(f.node, at + 1, status), lut);
        } else {
            C.d = ref;
        }
        C.o = offset_start_in(f.o, f.geo);
        C.magn = xmul(f.magn, m.tran);
        C.level = f.level + (spread ? 1 : 0);
    }
    C.node = tree_child(f.node, set, i);
    C.stage = kDistTrace;
}

// The counting pass of a reference-stream frame without diffuse rays: the
// pixel's ray tree (ray_trace_engine::ray_trace, raytracer.cc:20-87) walked
// post-order with an explicit stack, without shadow rays, counting the
// numbers the pixel draws in the reference's order (at each hit: the
// lights' rays, then the reflection set, then the refraction set; then the
// children's subtrees in order).
__device__ __forceinline__ uint32_t dist_count_pixel(const SceneView &sc, const CameraView &cam,
                                                     const LightSet &lights, const MaterialTable &table,
                                                     const DistLights &dl, const DistParams &dp,
                                                     const float *__restrict__ lut, DistStream &S, int x, int y,
                                                     DistFrame *F, uint32_t &status)
{
    uint32_t k = 0;
    const RayState cr = camera_ray(cam, x, y);
    F[0].o = cr.o;
    F[0].d = cr.d;
    F[0].magn = 1.0f;
    F[0].level = 0;
    F[0].node = kTreeRoot;
    F[0].stage = kDistTrace;
    int sp = 1;
    for (int step = 0; sp > 0 && step < dp.max_steps; ++step) {
        DistFrame &f = F[sp - 1];
        if (f.stage == kDistTrace) {
            HitRecord h;
            bool occ;
            status |= traverse<false>(sc, f.o, f.d, FLT_MAX, h, occ);
            f.nrefl = 0;
            f.nrefr = 0;
            f.stage = kDistDone;
            if (h.t < FLT_MAX) {
                const int32_t id = h.id - sc.tri_base;
                int32_t mi = sc.mat ? __ldg(&sc.mat[id]) : 0;
                if (mi < 0 || mi >= table.n) { status |= kStatusBadIndex; mi = 0; }
                const MaterialView &m = table.m[mi];
                RayState r;
                r.o = f.o;
                r.d = f.d;
                const SurfacePoint spt = surface_at(sc, r, h);
                const int lvl = min(f.level, kDistLevels - 1);
                for (int l = 0; l < lights.n; ++l) k += (uint32_t)dl.draws[l][lvl];
                f.o = spt.dst;
                f.sn = spt.sn;
                f.geo = spt.geo;
                f.mat = mi;
                f.out_in = spt.out_in ? 1 : 0;
                if ((double)xmul(f.magn, m.rf) > 0.1) {
                    f.nrefl = (dp.diffuse > 0 && dp.rfd[mi] != 0.0f) ? dist_count(dp.diffuse, f.level) : 1;
                    if (dp.diffuse > 0 && dp.rfd[mi] != 0.0f) { f.refl_at = k; k += 2u * (uint32_t)f.nrefl; }
                }
                if ((double)xmul(f.magn, m.tran) > 0.1) {
                    float ri = m.ri;
                    const float rdn = -xdot(f.d, f.sn);
                    if (f.out_in) ri = xdiv(1.0f, ri);
                    const float cos_t2 = xsub(1.0f, xmul(xmul(ri, ri), xsub(1.0f, xmul(rdn, rdn))));
                    if (!(cos_t2 < 0.0f)) {
                        f.nrefr = (dp.diffuse > 0 && dp.td[mi] != 0.0f) ? dist_count(dp.diffuse, f.level) : 1;
                        if (dp.diffuse > 0 && dp.td[mi] != 0.0f) { f.refr_at = k; k += 2u * (uint32_t)f.nrefr; }
                    }
                }
                f.child = 0;
                f.stage = kDistRefl;
            }
        }
        if (f.stage == kDistRefl) {
            if (f.child < f.nrefl) {
                if (sp >= kDistDepth) { status |= kStatusStepLimit; f.child = f.nrefl; continue; }
                spawn_child(f, table.m[f.mat], dp, 0, f.child, lut, S, status, F[sp]);
                ++f.child;
                ++sp;
                continue;
            }
            f.child = 0;
            f.stage = kDistRefr;
        }
        if (f.stage == kDistRefr) {
            if (f.child < f.nrefr) {
                if (sp >= kDistDepth) { status |= kStatusStepLimit; f.child = f.nrefr; continue; }
                spawn_child(f, table.m[f.mat], dp, 1, f.child, lut, S, status, F[sp]);
                ++f.child;
                ++sp;
                continue;
            }
            f.stage = kDistDone;
        }
        --sp;
    }
    if (sp > 0) status |= kStatusStepLimit;
    return k;
}

// How dist_walk walks: the whole tree from the camera ray; the camera ray's
// node alone (its colour from the lights and ka, its sets left in F[0] for
// the caller to hand out); or the subtree of a ray given in F[0].
enum : int { kDistWhole = 0, kDistRoot = 1, kDistSub = 2 };

// A pixel's ray tree shaded (ray_trace_engine::ray_trace, raytracer.cc:
// 20-87): the post-order walk of dist_count_pixel with every node shaded
// -- the coloured Phong of each light with its first ray's direction and
// length, weighted by the fraction of its rays that reach it (ray::find_rays
// ray.cc:91-104, light::find_rays light.h:62-164), plus ka; then each set's
// mean colour times rf, then tran -- drawing the numbers in the reference's
// order.  The walk is resumable: walk_advance moves it to the lane's next
// ray (a node's camera, mirror, refracted or diffuse ray: closest hit; a
// light's ray: any hit), the caller traces it, walk_consume takes the
// result -- so a warp's lanes trace together at one call site whatever
// stage their trees are at.  Walk holds the state besides the frame stack;
// the top frame's lights are shaded before any child is pushed, so one set
// of light state serves every frame.
struct Walk {
    int sp, step;
    float3 start, kd, ldir, c, out;
    float len;
    int light, sample, nl, made, lvl;
    uint32_t k;            // reference stream: the pixel's next number
    uint32_t kb, k0;       // the node's next number and its first
    uint32_t drawn, nsec;
    bool hit;
};

// A walk from the camera ray of (x, y), or (kDistSub) from the ray already
// in F[0].
template <int MODE>
__device__ __forceinline__ void walk_start(Walk &w, const CameraView &cam, DistFrame *F, int x, int y)
{
    if (MODE != kDistSub) {
        const RayState cr = camera_ray(cam, x, y);
        F[0].o = cr.o;
        F[0].d = cr.d;
        F[0].magn = 1.0f;
        F[0].level = 0;
        F[0].node = kTreeRoot;
        F[0].stage = kDistTrace;
    }
    w.sp = 1;
    w.step = 0;
    w.start = w.kd = w.ldir = w.c = make_float3(0.f, 0.f, 0.f);
    w.out = cam.background;
    w.len = 0.f;
    w.light = w.sample = w.made = w.lvl = 0;
    w.nl = 1;
    w.k = w.kb = w.k0 = w.drawn = w.nsec = 0;
    w.hit = false;
}

// Moves the walk to its next ray (true: ray in ro, rd, rt, any) or to its
// end (false: colour in w.out; kDistRoot: also when the camera ray's node
// is shaded, its sets left in F[0]).
template <int MODE>
__device__ __forceinline__ bool walk_advance(Walk &w, const SceneView &sc, const LightSet &lights,
                                             const MaterialTable &table, const DistLights &dl, const DistParams &dp,
                                             const int4 *__restrict__ area, const float *__restrict__ verts,
                                             const float *__restrict__ lut, DistStream &S, DistFrame *F,
                                             float3 &ro, float3 &rd, float &rt, bool &any, uint32_t &status)
{
    if (w.sp <= 0) return false;
    if (++w.step > dp.max_steps) {
        status |= kStatusStepLimit;
        w.sp = 0;
        return false;
    }
    for (int guard = 0; w.sp > 0 && guard < 4 * kDistDepth + 2 * RT_MAX_LIGHTS + 4; ++guard) {
        DistFrame &f = F[w.sp - 1];
        if (f.stage == kDistTrace) {
            ro = f.o;
            rd = f.d;
            rt = FLT_MAX;
            any = false;
            return true;
        }
        if (f.stage == kDistLights) {
            const MaterialView &m = table.m[f.mat];
            if (w.light < lights.n) {
                const LightView &L = lights.l[w.light];
                if (w.sample < w.nl) {
                    // ray `sample` of this light
                    float3 di;
                    float li;
                    if (w.nl == 1) {
                        shadow_ray(L, w.start, di, li);
                    } else if (dl.made[w.light][w.lvl] > 0) {
                        const float u0 = S.at(f.node, w.kb + 2 * w.sample, status);
                        const float u1 = S.at(f.node, w.kb + 2 * w.sample + 1, status);
                        area_ray(verts, sc.idx, __ldg(area + dl.first[w.light][w.lvl] + w.sample), w.start, u0, u1, di,
                                 li);
                    } else {
                        const float u0 = S.at(f.node, w.kb + 3 * w.sample, status);
                        const float u1 = S.at(f.node, w.kb + 3 * w.sample + 1, status);
                        const float u2 = S.at(f.node, w.kb + 3 * w.sample + 2, status);
                        soft_ray(L, lut, w.start, w.nl, w.sample, u0, u1, u2, di, li);
                    }
                    if (w.sample == 0) {
                        w.ldir = di;
                        w.len = li;
                    }
                    ro = w.start;
                    rd = di;
                    rt = li;
                    any = true;
                    return true;
                }
                w.kb += (uint32_t)dl.draws[w.light][w.lvl];
                w.nsec += (uint32_t)w.nl;
                phong_add<true>(L, m, w.kd, f.sn, f.d, w.ldir, w.len, xdiv((float)w.made, (float)w.nl), w.c);
                ++w.light;
                w.sample = 0;
                w.made = 0;
                if (w.light < lights.n)
                    w.nl = (lights.l[w.light].kind == RT_LIGHT_DIRECTIONAL) ? 1 : dist_count(dp.soft, f.level);
                continue;
            }
            // shaded: ka, then the sets (their numbers after the lights')
            f.c = xadd3(w.c, m.ka);
            if ((double)xmul(f.magn, m.rf) > 0.1) {
                if (dp.diffuse > 0 && dp.rfd[f.mat] != 0.0f) {
                    f.nrefl = dist_count(dp.diffuse, f.level);
                    f.refl_at = w.kb;
                    w.kb += 2u * (uint32_t)f.nrefl;
                } else {
                    f.nrefl = 1;
                }
            }
            if ((double)xmul(f.magn, m.tran) > 0.1) {
                float ri = m.ri;
                const float rdn = -xdot(f.d, f.sn);
                if (f.out_in) ri = xdiv(1.0f, ri);
                const float cos_t2 = xsub(1.0f, xmul(xmul(ri, ri), xsub(1.0f, xmul(rdn, rdn))));
                if (!(cos_t2 < 0.0f)) {
                    if (dp.diffuse > 0 && dp.td[f.mat] != 0.0f) {
                        f.nrefr = dist_count(dp.diffuse, f.level);
                        f.refr_at = w.kb;
                        w.kb += 2u * (uint32_t)f.nrefr;
                    } else {
                        f.nrefr = 1;
                    }
                }
            }
            w.drawn += w.kb - w.k0;
            if (!dp.pixel_stream) w.k = w.kb;
            f.child = 0;
            f.sum = make_float3(0.f, 0.f, 0.f);
            f.stage = kDistRefl;
            if (MODE == kDistRoot) {   // the camera ray's node alone: its sets stay in F[0]
                w.out = f.c;
                w.sp = 0;
                return false;
            }
            continue;
        }
        if (f.stage == kDistRefl) {
            const MaterialView &m = table.m[f.mat];
            if (f.child < f.nrefl) {
                if (w.sp >= kDistDepth) {
                    status |= kStatusStepLimit;
                    f.child = f.nrefl;
                } else {
                    spawn_child(f, m, dp, 0, f.child, lut, S, status, F[w.sp]);
                    ++f.child;
                    ++w.sp;
                }
            } else {
                if (m.rf > 0.0f && f.nrefl > 0) f.c = xadd3(f.c, xmul3(xdiv3(f.sum, (float)f.nrefl), m.rf));
                f.child = 0;
                f.sum = make_float3(0.f, 0.f, 0.f);
                f.stage = kDistRefr;
            }
            continue;
        }
        if (f.stage == kDistRefr) {
            const MaterialView &m = table.m[f.mat];
            if (f.child < f.nrefr) {
                if (w.sp >= kDistDepth) {
                    status |= kStatusStepLimit;
                    f.child = f.nrefr;
                } else {
                    spawn_child(f, m, dp, 1, f.child, lut, S, status, F[w.sp]);
                    ++f.child;
                    ++w.sp;
                }
            } else {
                if (m.tran > 0.0f && f.nrefr > 0) f.c = xadd3(f.c, xmul3(xdiv3(f.sum, (float)f.nrefr), m.tran));
                f.stage = kDistDone;
            }
            continue;
        }
        // done: the frame's colour goes to its parent's current set
        const float3 col = f.c;
        --w.sp;
        if (w.sp == 0) w.out = col;
        else F[w.sp - 1].sum = xadd3(F[w.sp - 1].sum, col);
    }
    if (w.sp > 0) {   // never expected: the guard bounds the moves between two rays
        status |= kStatusStepLimit;
        w.sp = 0;
    }
    return false;
}

// Takes the result of the ray walk_advance asked for.
template <int MODE>
__device__ __forceinline__ void walk_consume(Walk &w, const Trav &T, bool any, const SceneView &sc,
                                             const CameraView &cam, const LightSet &lights, const MaterialTable &table,
                                             const DistParams &dp, DistFrame *F, uint32_t &status)
{
    DistFrame &f = F[w.sp - 1];
    if (any) {
        if (!T.occluded) ++w.made;
        ++w.sample;
        return;
    }
    // the node's closest hit
    if (w.sp > 1 || MODE == kDistSub) ++w.nsec;
    f.nrefl = 0;
    f.nrefr = 0;
    if (!(T.hit.t < FLT_MAX)) {
        f.c = cam.background;
        f.stage = kDistDone;
        if (MODE == kDistRoot) {
            w.out = f.c;
            w.sp = 0;
        }
        return;
    }
    const int32_t id = T.hit.id - sc.tri_base;
    if (w.sp == 1 && MODE != kDistSub) w.hit = true;
    int32_t mi = sc.mat ? __ldg(&sc.mat[id]) : 0;
    if (mi < 0 || mi >= table.n) { status |= kStatusBadIndex; mi = 0; }
    const MaterialView &m = table.m[mi];
    RayState r;
    r.o = f.o;
    r.d = f.d;
    const SurfacePoint spt = surface_at(sc, r, T.hit);
    w.start = offset_start(spt.dst, spt.geo);
    w.kd = material_kd(m, spt);
    w.c = make_float3(0.f, 0.f, 0.f);
    w.lvl = min(f.level, kDistLevels - 1);
    // this node's first number: its own stream's first, or the pixel's next
    // in the reference's stream
    w.k0 = dp.pixel_stream ? 0u : w.k;
    w.kb = w.k0;
    w.light = 0;
    w.sample = 0;
    w.made = 0;
    w.nl = (lights.n > 0 && lights.l[0].kind == RT_LIGHT_DIRECTIONAL) ? 1 : dist_count(dp.soft, f.level);
    f.o = spt.dst;
    f.sn = spt.sn;
    f.geo = spt.geo;
    f.mat = mi;
    f.out_in = spt.out_in ? 1 : 0;
    f.stage = kDistLights;
}

// The whole walk of one lane (its lanes' rays traced together while their
// walks last).
template <int MODE>
__device__ __forceinline__ uint32_t dist_walk(const SceneView &sc, const CameraView &cam, const LightSet &lights,
                                              const MaterialTable &table, const DistLights &dl, const DistParams &dp,
                                              const int4 *__restrict__ area, const float *__restrict__ verts,
                                              const float *__restrict__ lut, DistStream &S, int x, int y,
                                              DistFrame *F, float3 &out, bool &hit, uint32_t &nsec,
                                              uint32_t &status)
{
    Walk w;
    walk_start<MODE>(w, cam, F, x, y);
    uint2 stack[kStackSize];
    for (;;) {
        float3 ro, rd;
        float rt;
        bool any;
        if (!walk_advance<MODE>(w, sc, lights, table, dl, dp, area, verts, lut, S, F, ro, rd, rt, any, status)) break;
        Trav T;
        trav_begin(T, sc, ro, rd, rt, any);
        while (!trav_step<false>(T, stack, sc, any, status, nullptr)) {
        }
        walk_consume<MODE>(w, T, any, sc, cam, lights, table, dp, F, status);
    }
    out = w.out;
    hit = w.hit;
    nsec += w.nsec;
    return w.drawn;
}

// One launch of the distributed walk: the counting pass (SHADE false:
// counts[pix] = numbers the pixel draws) or the shading pass (numbers from
// the pixels' own streams, or from rnd at prefix[pix]).  A warp walks the 32
// pixels of an 8x4 tile, its lanes' rays traced together.
// RT_DIST_MIN_BLOCKS: resident blocks per SM the register allocation must
// allow (5: 96 registers, measured fastest for the converged walk; 4 was
// for the walk that traced at three call sites).
#ifndef RT_DIST_MIN_BLOCKS
#define RT_DIST_MIN_BLOCKS 5
#endif
template <bool SHADE>
__global__ void __launch_bounds__(kTraceThreads, RT_DIST_MIN_BLOCKS) k_dist(SceneView sc, CameraView cam, LightSet lights,
                                                        MaterialTable table, DistLights dl, DistParams dp,
                                                        const int4 *__restrict__ area, const float *__restrict__ verts,
                                                        const float *__restrict__ lut, const float *__restrict__ rnd,
                                                        int64_t nrnd, const int64_t *__restrict__ prefix,
                                                        int64_t *__restrict__ counts, uint8_t *__restrict__ rgb,
                                                        float *__restrict__ fimg, Counters *ctr)
{
    DistFrame F[kDistDepth];
    int tiles_x;
    const int items = tiles_of<8>(cam.xres, cam.yres, tiles_x) * 32;
    uint32_t status = 0;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel<8>(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
        uint32_t nsec = 0, drawn = 0;
        bool hit = false;
        if (live) {
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            DistStream S;
            S.win = rnd;
            S.nwin = nrnd;
            S.base = (SHADE && !dp.pixel_stream) ? prefix[pix] : 0;
            S.pixel = (uint32_t)pix;
            S.key0 = dp.key0;
            S.key1 = dp.key1;
            S.pixel_mode = dp.pixel_stream != 0;
            S.blk = 0xffffffffu;
            S.bnode = 0;
            float3 c;
            if (SHADE)
                drawn = dist_walk<kDistWhole>(sc, cam, lights, table, dl, dp, area, verts, lut, S, x, y, F, c, hit,
                                              nsec, status);
            else
                drawn = dist_count_pixel(sc, cam, lights, table, dl, dp, lut, S, x, y, F, status);
            if (SHADE) {
                if (rgb) store_rgb(rgb, pix, c);
                if (fimg) {
                    fimg[3 * pix] = c.x;
                    fimg[3 * pix + 1] = c.y;
                    fimg[3 * pix + 2] = c.z;
                }
            } else {
                counts[pix] = (int64_t)drawn;
            }
        }
        if (SHADE) {
            warp_count(&ctr->primary, live);
            warp_count(&ctr->hits, hit);
            warp_add(&ctr->secondary, nsec);
            unsigned long long d = drawn;
            for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
            if ((threadIdx.x & 31) == 0 && d) atomicAdd(&ctr->drawn, d);
        }
    }
    if (status) atomicOr(&ctr->status, status);
}

// Frames of per-pixel streams with ray trees are traced in three launches:
// the camera ray's node of every pixel (k_dist_root: its colour from the
// lights and ka, its sets' rays handed out as separate items), every item's
// subtree (k_dist_sub), then every pixel's colour from its node's and its
// items' (k_dist_combine, in the walk's order of additions).  A node's
// numbers are keyed by the node, so an item's subtree draws the same numbers
// traced alone as in the pixel's walk, and neighbouring items -- the rays of
// one set -- trace together.
struct DistItem {
    float4 o_magn;       // origin, power
    float4 d_level;      // direction, componant level (int bits)
    ulonglong2 node;     // tree node, pixel
};

__device__ __forceinline__ DistStream pixel_streams(const DistParams &dp, uint32_t pix)
{
    DistStream S;
    S.win = nullptr;
    S.nwin = 0;
    S.base = 0;
    S.pixel = pix;
    S.key0 = dp.key0;
    S.key1 = dp.key1;
    S.pixel_mode = true;
    S.blk = 0xffffffffu;
    S.bnode = 0;
    return S;
}

__global__ void __launch_bounds__(kTraceThreads, RT_DIST_MIN_BLOCKS) k_dist_root(
    SceneView sc, CameraView cam, LightSet lights, MaterialTable table, DistLights dl, DistParams dp,
    const int4 *__restrict__ area, const float *__restrict__ verts, const float *__restrict__ lut,
    float4 *__restrict__ root_c, int4 *__restrict__ root_sets, DistItem *__restrict__ items, int32_t cap,
    int32_t *__restrict__ nitems, Counters *ctr)
{
    DistFrame F[kDistDepth];   // the walk stops at F[0]
    int tiles_x;
    const int items_n = tiles_of<8>(cam.xres, cam.yres, tiles_x) * 32;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t status = 0;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items_n) break;
        int x, y;
        tile_pixel<8>(base + (int)lane, tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
        uint32_t nsec = 0, drawn = 0;
        bool hit = false;
        float3 c = cam.background;
        int cnt = 0;
        const size_t pix = live ? (size_t)x + (size_t)y * (size_t)cam.xres : 0;
        if (live) {
            DistStream S = pixel_streams(dp, (uint32_t)pix);
            drawn = dist_walk<kDistRoot>(sc, cam, lights, table, dl, dp, area, verts, lut, S, x, y, F, c, hit,
                                                nsec, status);
            if (F[0].stage == kDistRefl) cnt = F[0].nrefl + F[0].nrefr;
        }
        // the warp's items in lane order, reflection and refraction sets in
        // lists of their own (a warp of subtrees then holds one kind), one
        // allocation per list per warp
        const int nr = cnt > 0 ? F[0].nrefl : 0, nt = cnt > 0 ? F[0].nrefr : 0;
        int ir = nr, it_ = nt;
        for (int o = 1; o < 32; o <<= 1) {
            const int vr = __shfl_up_sync(0xffffffffu, ir, o), vt = __shfl_up_sync(0xffffffffu, it_, o);
            if ((int)lane >= o) { ir += vr; it_ += vt; }
        }
        int rbase = 0, tbase = 0;
        if (lane == 31u) {
            if (ir) rbase = atomicAdd(&nitems[0], ir);
            if (it_) tbase = atomicAdd(&nitems[1], it_);
        }
        rbase = __shfl_sync(0xffffffffu, rbase, 31) + ir - nr;
        tbase = __shfl_sync(0xffffffffu, tbase, 31) + it_ - nt;
        if (live) {
            // else the host grows the lists and runs again
            const bool fits = rbase >= 0 && rbase + nr <= cap && tbase >= 0 && tbase + nt <= cap;
            if (cnt > 0 && fits) {
                DistStream S = pixel_streams(dp, (uint32_t)pix);
                const MaterialView &m = table.m[F[0].mat];
                for (int j = 0; j < cnt; ++j) {
                    const int set = j < nr ? 0 : 1;
                    DistFrame C;
                    spawn_child(F[0], m, dp, set, set ? j - nr : j, lut, S, status, C);
                    DistItem it;
                    it.o_magn = make_float4(C.o.x, C.o.y, C.o.z, C.magn);
                    it.d_level = make_float4(C.d.x, C.d.y, C.d.z, __int_as_float(C.level));
                    it.node = make_ulonglong2(C.node, (unsigned long long)pix);
                    items[set ? (size_t)cap + tbase + (j - nr) : (size_t)rbase + j] = it;
                }
            }
            root_c[pix] = make_float4(c.x, c.y, c.z, __int_as_float(cnt > 0 ? F[0].mat : 0));
            root_sets[pix] = make_int4(rbase, nr, tbase, nt);
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, hit);
        warp_add(&ctr->secondary, nsec);
        unsigned long long d = drawn;
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if (lane == 0u && d) atomicAdd(&ctr->drawn, d);
    }
    if (status) atomicOr(&ctr->status, status);
}

// The items' subtrees, one per lane; a warp takes 32 consecutive items
// (the rays of one or two sets) at a time.  (Lanes that take the next item
// as soon as theirs is finished were measured slower: 61 against 41 ms on
// the 512x512 glass frame with 16-ray diffuse sets, their rays no longer
// neighbours.)
// 6 resident blocks (80 registers): 34.1 ms against 41.3 at 4 and 37.1 at 5
// on the 512x512 glass frame with 16-ray diffuse sets; 7 and 8 no faster
#ifndef RT_DIST_SUB_MIN_BLOCKS
#define RT_DIST_SUB_MIN_BLOCKS 6
#endif
__global__ void __launch_bounds__(kTraceThreads, RT_DIST_SUB_MIN_BLOCKS) k_dist_sub(
    SceneView sc, CameraView cam, LightSet lights, MaterialTable table, DistLights dl, DistParams dp,
    const int4 *__restrict__ area, const float *__restrict__ verts, const float *__restrict__ lut,
    const DistItem *__restrict__ items, int32_t nr, int32_t nt, int32_t cap, float4 *__restrict__ item_c,
    Counters *ctr)
{
    DistFrame F[kDistDepth];
    const uint32_t lane = threadIdx.x & 31u;
    // the reflection list's items, then (from a warp boundary on) the
    // refraction list's
    const int rw = (nr + 31) & ~31;
    const int n = rw + nt;
    uint32_t status = 0;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= n) break;
        const int v = base + (int)lane;
        const int i = v < rw ? (v < nr ? v : -1) : (v - rw < nt ? cap + (v - rw) : -1);
        uint32_t nsec = 0, drawn = 0;
        if (i >= 0) {
            const DistItem it = items[i];
            F[0].o = make_float3(it.o_magn.x, it.o_magn.y, it.o_magn.z);
            F[0].magn = it.o_magn.w;
            F[0].d = make_float3(it.d_level.x, it.d_level.y, it.d_level.z);
            F[0].level = __float_as_int(it.d_level.w);
            F[0].node = it.node.x;
            F[0].stage = kDistTrace;
            DistStream S = pixel_streams(dp, (uint32_t)it.node.y);
            float3 c;
            bool hit;
            drawn = dist_walk<kDistSub>(sc, cam, lights, table, dl, dp, area, verts, lut, S, 0, 0, F, c, hit, nsec,
                                        status);
            item_c[i] = make_float4(c.x, c.y, c.z, 0.f);
        }
        warp_add(&ctr->secondary, nsec);
        unsigned long long d = drawn;
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if (lane == 0u && d) atomicAdd(&ctr->drawn, d);
    }
    if (status) atomicOr(&ctr->status, status);
}

// A pixel's colour: its node's, then each set's mean added times rf, then
// tran (the walk's additions, in its order).
__global__ void k_dist_combine(CameraView cam, MaterialTable table, const float4 *__restrict__ root_c,
                               const int4 *__restrict__ root_sets, const float4 *__restrict__ item_c, int32_t nr,
                               int32_t nt, int32_t cap, uint8_t *__restrict__ rgb, float *__restrict__ fimg,
                               Counters *ctr)
{
    const int32_t npix = cam.xres * cam.yres;
    uint32_t status = 0;
    for (int32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const float4 r = root_c[p];
        const int4 sets = root_sets[p];   // reflection list's first, count; refraction list's first, count
        float3 c = make_float3(r.x, r.y, r.z);
        if (sets.y + sets.w > 0) {
            if (sets.x < 0 || sets.x + sets.y > nr || sets.z < 0 || sets.z + sets.w > nt) {
                status |= kStatusBadIndex;
            } else {
                const MaterialView &m = table.m[__float_as_int(r.w)];
                float3 sum = make_float3(0.f, 0.f, 0.f);
                for (int j = 0; j < sets.y; ++j) {
                    const float4 q = item_c[sets.x + j];
                    sum = xadd3(sum, make_float3(q.x, q.y, q.z));
                }
                if (m.rf > 0.0f && sets.y > 0) c = xadd3(c, xmul3(xdiv3(sum, (float)sets.y), m.rf));
                sum = make_float3(0.f, 0.f, 0.f);
                for (int j = 0; j < sets.w; ++j) {
                    const float4 q = item_c[(size_t)cap + sets.z + j];
                    sum = xadd3(sum, make_float3(q.x, q.y, q.z));
                }
                if (m.tran > 0.0f && sets.w > 0) c = xadd3(c, xmul3(xdiv3(sum, (float)sets.w), m.tran));
            }
        }
        if (rgb) store_rgb(rgb, (size_t)p, c);
        if (fimg) {
            fimg[3 * (size_t)p] = c.x;
            fimg[3 * (size_t)p + 1] = c.y;
            fimg[3 * (size_t)p + 2] = c.z;
        }
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

rt_status check_shapes(const rt_scene *s, const rt_light *lights, int32_t nlights, const rt_light_shape *shapes,
                       const char *who);
rt_status stream_window(SoftState &S, int64_t offset, int64_t total, cudaStream_t st, const float **rnd);

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
    {
        const rt_status st = check_shapes(s, lights, nlights, shapes, "rt_render_soft_shadows");
        if (st != RT_OK) return st;
    }
    if (!s->built) return sfail(RT_ERR_NOT_BUILT, "rt_render_soft_shadows: hierarchy not built");
    if (s->mat_max >= nmaterials)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_soft_shadows: the scene's material indices exceed the table");
    rt_context *ctx = s->ctx;
    SGuard g(ctx->device);
    if (!ctx->soft) {
        ctx->soft = new (std::nothrow) SoftState();
        if (!ctx->soft) return sfail(RT_ERR_OUT_OF_MEMORY, "rt_render_soft_shadows: state allocation");
        ctx->soft->device = ctx->device;
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
    // the frame's slice of the reference's stream
    const float *rnd = nullptr;
    {
        const rt_status wst = stream_window(S, stream_offset, total, st, &rnd);
        if (wst != RT_OK) return wst;
    }

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

namespace {

int sub_blocks_per_sm()
{
    static const int per_sm = [] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_dist_sub, kTraceThreads, 0) != cudaSuccess || b < 1) {
            cudaGetLastError();
            b = 2;
        }
        return b;
    }();
    return per_sm;
}

int dist_blocks_per_sm()
{
    static const int per_sm = [] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_dist<true>, kTraceThreads, 0) != cudaSuccess || b < 1) {
            cudaGetLastError();
            b = 2;
        }
        return b;
    }();
    return per_sm;
}

// Worst-case ray tree of a distributed frame: a ray of power a^i * b^j
// (a, b the largest rf and tran of the table) at componant level k spawns,
// while the child's power exceeds 0.1, a reflection set -- one mirror ray,
// or max(diffuse / 4^k, 1) rays at level k + 1 where some reflective
// material spreads -- and likewise a refraction set.  rays: the largest
// tree; depth: its levels below the camera ray; levels: the deepest
// componant level.
struct TreeBound {
    double rays = 0.0;
    int depth = 0, levels = 0;
};

struct TreeBounder {
    double a, b;
    bool mirror_r, spread_r, mirror_t, spread_t;
    int diffuse;
    static constexpr int kI = 4 * RT_MAX_BOUNCES + 2, kK = 18;
    std::vector<double> memo;
    std::vector<int> deep, lev;

    TreeBounder() : memo((size_t)kI * kI * kK, -1.0), deep((size_t)kI * kI * kK, 0), lev((size_t)kI * kI * kK, 0) {}

    // rays of the worst tree below a ray of power a^i b^j at level k
    double f(int i, int j, int k)
    {
        const size_t at = ((size_t)i * kI + (size_t)j) * kK + (size_t)k;
        if (memo[at] >= 0.0) return memo[at];
        const double thr = 0.1 * (1.0 - 1.0e-5);
        double r = 1.0;
        int d = 0, l = k;
        for (int side = 0; side < 2; ++side) {
            const int ni = i + (side == 0), nj = j + (side == 1);
            if (ni + nj >= kI - 1 || !(std::pow(a, ni) * std::pow(b, nj) > thr)) continue;
            const bool mirror = side == 0 ? mirror_r : mirror_t, spread = side == 0 ? spread_r : spread_t;
            double best = 0.0;
            if (mirror) {
                best = f(ni, nj, k);
                const size_t c = ((size_t)ni * kI + (size_t)nj) * kK + (size_t)k;
                d = std::max(d, 1 + deep[c]);
                l = std::max(l, lev[c]);
            }
            if (spread) {
                const int kk = std::min(k + 1, kK - 1);
                const double nr = (double)std::max(diffuse >> (2 * std::min(k, kDistLevels - 1)), 1);
                best = std::max(best, nr * f(ni, nj, kk));
                const size_t c = ((size_t)ni * kI + (size_t)nj) * kK + (size_t)kk;
                d = std::max(d, 1 + deep[c]);
                l = std::max(l, lev[c]);
            }
            r += best;
        }
        memo[at] = r;
        deep[at] = d;
        lev[at] = l;
        return r;
    }
};

TreeBound dist_tree_bound(const rt_material *m, int32_t n, int32_t diffuse)
{
    TreeBounder tb;
    tb.a = tb.b = 0.0;
    tb.mirror_r = tb.spread_r = tb.mirror_t = tb.spread_t = false;
    tb.diffuse = diffuse;
    for (int32_t i = 0; i < n; ++i) {
        tb.a = std::max(tb.a, (double)m[i].rf);
        tb.b = std::max(tb.b, (double)m[i].tran);
        if (m[i].rf > 0.0f) {
            if (diffuse > 0 && m[i].rfd != 0.0f) tb.spread_r = true;
            else tb.mirror_r = true;
        }
        if (m[i].tran > 0.0f) {
            if (diffuse > 0 && m[i].td != 0.0f) tb.spread_t = true;
            else tb.mirror_t = true;
        }
    }
    TreeBound out;
    out.rays = tb.f(0, 0, 0);
    out.depth = tb.deep[0];
    out.levels = tb.lev[0];
    return out;
}

// Shapes of the lights (rt_light_shape): radii finite and >= 0; triangle
// lists in range on point or spot lights of radius 0.
rt_status check_shapes(const rt_scene *s, const rt_light *lights, int32_t nlights, const rt_light_shape *shapes,
                       const char *who)
{
    for (int32_t i = 0; i < nlights && shapes; ++i) {
        const rt_light_shape &sh = shapes[i];
        const std::string w(who);
        if (!(sh.radius >= 0.0f && sh.radius < 3.0e38f))
            return sfail(RT_ERR_INVALID_ARG, (w + ": light radius must be finite and >= 0").c_str());
        if (sh.ntris < 0 || (sh.ntris > 0 && !sh.tris))
            return sfail(RT_ERR_INVALID_ARG, (w + ": bad triangle list of a light").c_str());
        if (sh.ntris > 0 && (sh.radius != 0.0f || (lights[i].kind & 0xff) == RT_LIGHT_DIRECTIONAL))
            return sfail(RT_ERR_INVALID_ARG,
                         (w + ": a triangle-defined light is a point or spot light of radius 0").c_str());
        for (int32_t j = 0; j < sh.ntris; ++j)
            if (sh.tris[j] < 0 || sh.tris[j] >= s->ntris)
                return sfail(RT_ERR_INVALID_ARG, (w + ": light triangle index out of range").c_str());
    }
    return RT_OK;
}

// The frame's numbers [offset, offset + total) of the reference's stream on
// the device (generated on the host into pinned memory, copied over), kept
// while later frames fall inside them; *rnd points at number offset.  A
// frame that starts where the last one ended finds its numbers already
// generated by the read-ahead (or the read-ahead still running: it is
// joined).
rt_status stream_window(SoftState &S, int64_t offset, int64_t total, cudaStream_t st, const float **rnd)
{
    *rnd = nullptr;
    if (total <= 0) return RT_OK;
    if (S.win_base >= 0 && offset >= S.win_base && offset + total <= S.win_base + S.win_len) {
        *rnd = (const float *)S.window.ptr + (offset - S.win_base);
        return RT_OK;
    }
    join_ahead(S);
    const int64_t want = total + total / 4;   // read-ahead length: the next frame draws about as many
    if (!(S.stage_base >= 0 && offset >= S.stage_base && offset + total <= S.stage_base + S.stage_len)) {
        // not read ahead: generate the slice here
        // the last upload reads the staging buffer: it must be done first
        RT_CUDA_S(cudaStreamSynchronize(st), "synchronize");
        if (S.staging_cap < (size_t)want) {
            if (S.staging) cudaFreeHost(S.staging);
            S.staging = nullptr;
            S.staging_cap = 0;
            S.stage_base = -1;
            S.stage_len = 0;
            RT_CUDA_S(cudaMallocHost(&S.staging, (size_t)want * sizeof(float)), "pinned stream staging");
            S.staging_cap = (size_t)want;
        }
        S.stage_base = -1;
        S.stage_len = 0;
        try {
            generate_slice(S.rng, offset, total, S.staging);
        } catch (...) {
            return sfail(RT_ERR_OUT_OF_MEMORY, "random stream: host memory for the slice's generator states");
        }
        S.stage_base = offset;
        S.stage_len = total;
    }
    RT_CUDA_S(S.window.reserve((size_t)total * sizeof(float)), "stream allocation");
    RT_CUDA_S(cudaMemcpyAsync(S.window.ptr, S.staging + (offset - S.stage_base), (size_t)total * sizeof(float),
                              cudaMemcpyHostToDevice, st),
              "stream copy");
    if (!S.copied) RT_CUDA_S(cudaEventCreateWithFlags(&S.copied, cudaEventDisableTiming), "event creation");
    RT_CUDA_S(cudaEventRecord(S.copied, st), "event record");
    S.win_base = offset;
    S.win_len = total;
    *rnd = (const float *)S.window.ptr;
    // read ahead [offset + total, offset + total + want): the numbers already
    // generated past the frame move to the front of staging (once the
    // upload is done), the rest continue from rng, which stands at their end
    if ((size_t)want <= S.staging_cap) {
        const int64_t next = offset + total;
        SoftState *P = &S;
        try {
            S.ahead = std::thread([P, next, want] {
                cudaSetDevice(P->device);
                if (cudaEventSynchronize(P->copied) != cudaSuccess) {
                    P->stage_base = -1;   // nothing kept: the next window generates its own
                    P->stage_len = 0;
                    return;
                }
                const int64_t keep = P->stage_base + P->stage_len - next;
                if (keep > 0)
                    std::memmove(P->staging, P->staging + (next - P->stage_base), (size_t)keep * sizeof(float));
                const int64_t kept = std::max<int64_t>(keep, 0);
                try {
                    if (want > kept) generate_slice(P->rng, next + kept, want - kept, P->staging + kept);
                    P->stage_base = next;
                    P->stage_len = std::max(kept, want);
                } catch (...) {   // out of host memory: keep what is there
                    P->stage_base = kept > 0 ? next : -1;
                    P->stage_len = kept;
                }
            });
        } catch (...) {   // no thread: the next window generates its own numbers
        }
    }
    return RT_OK;
}

}  // namespace

extern "C" rt_status rt_render_distributed(rt_scene *s, const rt_camera *camera, const rt_light *lights,
                                           int32_t nlights, const rt_light_shape *shapes,
                                           const rt_material *materials, int32_t nmaterials,
                                           const rt_sampling *sampling, uint8_t *rgb_out, float *rgb_f32,
                                           int64_t *stream_end, rt_render_stats *stats)
{
    if (!s || !camera || !materials || !sampling || (!rgb_out && !rgb_f32))
        return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: NULL argument");
    if (camera->xres <= 0 || camera->yres <= 0 || (int64_t)camera->xres * camera->yres > (int64_t)1 << 28)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: camera resolution out of range");
    if (nlights < 0 || nlights > RT_MAX_LIGHTS || (nlights > 0 && !lights))
        return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: light count out of range");
    if (nmaterials < 1 || nmaterials > RT_MAX_MATERIALS)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: material count must be 1..RT_MAX_MATERIALS");
    const rt_sampling smp = *sampling;
    if (smp.soft_samples < 1 || smp.soft_samples > RT_MAX_SOFT_SAMPLES || smp.diffuse_samples < 0 ||
        smp.diffuse_samples > RT_MAX_SOFT_SAMPLES)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: sample counts out of range");
    if (smp.stream != RT_STREAM_REFERENCE && smp.stream != RT_STREAM_PIXEL)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: unknown stream");
    if (smp.stream == RT_STREAM_REFERENCE && smp.stream_offset < 0)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: negative stream offset");
    bool tree = false, spread = false;
    for (int32_t i = 0; i < nmaterials; ++i) {
        const rt_material &m = materials[i];
        if (!(m.rf >= 0.0f && m.rf < 1.0f) || !(m.tran >= 0.0f && m.tran < 1.0f))
            return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: reflectivity and transparency must be in [0, 1)");
        if (m.tran > 0.0f && !(m.ri > 0.0f && m.ri < 3.0e38f))
            return sfail(RT_ERR_INVALID_ARG,
                         "rt_render_distributed: a transparent material needs a finite positive refractive index");
        if (!(std::fabs(m.rfd) < 3.0e38f) || !(std::fabs(m.td) < 3.0e38f))
            return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: diffuse spreads must be finite");
        tree = tree || m.rf > 0.0f || m.tran > 0.0f;
        spread = spread || (smp.diffuse_samples > 0 && ((m.rf > 0.0f && m.rfd != 0.0f) || (m.tran > 0.0f && m.td != 0.0f)));
    }
    if (spread && smp.stream == RT_STREAM_REFERENCE)
        return sfail(RT_ERR_INVALID_ARG,
                     "rt_render_distributed: diffuse rays draw the reference's stream in an order one pass cannot "
                     "replay in parallel (a pixel's count depends on where earlier random rays landed); use "
                     "RT_STREAM_PIXEL");
    {
        const rt_status st = check_shapes(s, lights, nlights, shapes, "rt_render_distributed");
        if (st != RT_OK) return st;
    }
    if (!s->built) return sfail(RT_ERR_NOT_BUILT, "rt_render_distributed: hierarchy not built");
    if (s->mat_max >= nmaterials)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: the scene's material indices exceed the table");
    // without ray trees or diffuse rays, the reference-stream frame is the
    // soft-shadow frame
    if (!tree && smp.stream == RT_STREAM_REFERENCE)
        return rt_render_soft_shadows(s, camera, lights, nlights, shapes, materials, nmaterials, smp.soft_samples,
                                      smp.stream_offset, rgb_out, rgb_f32, stream_end, stats);
    const TreeBound tb = dist_tree_bound(materials, nmaterials, smp.diffuse_samples);
    if (tb.depth > RT_MAX_BOUNCES || tb.rays > (double)RT_MAX_TREE_RAYS || tb.levels > 15)
        return sfail(RT_ERR_INVALID_ARG, "rt_render_distributed: the materials allow more than RT_MAX_BOUNCES levels "
                                         "or RT_MAX_TREE_RAYS rays per pixel");

    rt_context *ctx = s->ctx;
    SGuard g(ctx->device);
    if (!ctx->soft) {
        ctx->soft = new (std::nothrow) SoftState();
        if (!ctx->soft) return sfail(RT_ERR_OUT_OF_MEMORY, "rt_render_distributed: state allocation");
        ctx->soft->device = ctx->device;
    }
    SoftState &S = *ctx->soft;
    cudaStream_t st = ctx->stream;
    if (!S.lut_ready) {
        std::vector<float> lut(kCosLutSize);
        for (int i = 0; i < kCosLutSize; ++i)
            lut[i] = (float)std::cos((double)((((float)i * 2.0f) * kRefPi) / (float)kCosLutSize));
        RT_CUDA_S(S.lut.reserve(kCosLutSize * sizeof(float)), "cosine table allocation");
        RT_CUDA_S(cudaMemcpy(S.lut.ptr, lut.data(), kCosLutSize * sizeof(float), cudaMemcpyHostToDevice),
                  "cosine table copy");
        S.lut_ready = true;
    }
    // lights: per componant level, the rays of every triangle-defined
    // light and the numbers a hit draws
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = 0;
    DistLights dl = {};
    std::vector<int4> area_rays;
    for (int i = 0; i < nlights; ++i) {
        ls.l[i] = make_light_view(lights[i]);
        ls.l[i].radius = shapes ? shapes[i].radius : 0.0f;
        if (ls.l[i].kind == RT_LIGHT_DIRECTIONAL) continue;
        for (int k = 0; k < kDistLevels; ++k) {
            const int32_t n = std::max(smp.soft_samples >> (2 * k), 1);
            if (n == 1) continue;
            if (shapes && shapes[i].ntris > 0) {
                const int32_t nt = shapes[i].ntris;
                std::vector<int32_t> cnt((size_t)nt);
                const int32_t made = area_light_rays(nt, n, cnt.data());
                if (made < n)
                    return sfail(RT_ERR_INVALID_ARG,
                                 "rt_render_distributed: a triangle-defined light makes fewer rays than asked");
                dl.first[i][k] = (int32_t)area_rays.size();
                dl.made[i][k] = made;
                dl.draws[i][k] = 2 * made;
                for (int32_t j = 0; j < nt; ++j)
                    for (int32_t q = 0; q < cnt[(size_t)j]; ++q)
                        area_rays.push_back(make_int4(shapes[i].tris[j], cnt[(size_t)j], q, 0));
            } else {
                dl.draws[i][k] = 3 * n;
            }
        }
    }
    if (!area_rays.empty()) {
        RT_CUDA_S(S.area.reserve(area_rays.size() * sizeof(int4)), "light ray table allocation");
        RT_CUDA_S(cudaMemcpyAsync(S.area.ptr, area_rays.data(), area_rays.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                  st),
                  "light ray table copy");
    }
    MaterialTable mt;
    mt.n = nmaterials;
    DistParams dp = {};
    dp.soft = smp.soft_samples;
    dp.diffuse = smp.diffuse_samples;
    dp.pixel_stream = smp.stream == RT_STREAM_PIXEL ? 1 : 0;
    dp.key0 = (uint32_t)smp.seed;
    dp.key1 = (uint32_t)(smp.seed >> 32);
    // walk steps per pixel: every ray of the tree and every light's rays at each of its hits
    dp.max_steps = (int32_t)std::min(8.0 * tb.rays * (1.0 + (double)nlights * smp.soft_samples) + 64.0, 1.0e9);
    for (int i = 0; i < nmaterials; ++i) {
        mt.m[i] = make_material_view(materials[i]);
        dp.rfd[i] = materials[i].rfd;
        dp.td[i] = materials[i].td;
    }
    const SceneView sv = scene_view(s);
    const CameraView cv = make_camera_view(*camera);
    const size_t npix = (size_t)camera->xres * (size_t)camera->yres;
    const int grid = dist_blocks_per_sm() * ctx->sm_count;

    RT_CUDA_S(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), st), "counter clear");
    RT_CUDA_S(cudaEventRecord(ctx->ev0, st), "event record");
    const float *rnd = nullptr;
    int64_t total = 0;
    if (smp.stream == RT_STREAM_REFERENCE) {
        // counting pass, scan, the frame's slice of the stream
        RT_CUDA_S(S.counts.reserve(npix * sizeof(int64_t)), "count allocation");
        RT_CUDA_S(S.prefix64.reserve(npix * sizeof(int64_t)), "prefix allocation");
        size_t scan_bytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (const int64_t *)S.counts.ptr, (int64_t *)S.prefix64.ptr,
                                      (int)npix, st);
        RT_CUDA_S(S.scan64_temp.reserve(scan_bytes), "scan scratch allocation");
        k_dist<false><<<grid, kTraceThreads, 0, st>>>(sv, cv, ls, mt, dl, dp, (const int4 *)S.area.ptr, s->d_verts,
                                                      (const float *)S.lut.ptr, nullptr, 0, nullptr,
                                                      (int64_t *)S.counts.ptr, nullptr, nullptr, ctx->d_counters);
        RT_CUDA_S(cudaGetLastError(), "counting launch");
        cub::DeviceScan::ExclusiveSum(S.scan64_temp.ptr, scan_bytes, (const int64_t *)S.counts.ptr,
                                      (int64_t *)S.prefix64.ptr, (int)npix, st);
        RT_CUDA_S(cudaGetLastError(), "scan launch");
        int64_t last[2];
        RT_CUDA_S(cudaMemcpyAsync(&last[0], (const int64_t *)S.prefix64.ptr + (npix - 1), sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, st),
                  "prefix read");
        RT_CUDA_S(cudaMemcpyAsync(&last[1], (const int64_t *)S.counts.ptr + (npix - 1), sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, st),
                  "count read");
        RT_CUDA_S(cudaStreamSynchronize(st), "synchronize");
        total = last[0] + last[1];
        const rt_status wst = stream_window(S, smp.stream_offset, total, st, &rnd);
        if (wst != RT_OK) return wst;
        RT_CUDA_S(cudaMemsetAsync(&ctx->d_counters->work, 0, sizeof(int), st), "work counter clear");
    }
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
    // per-pixel streams with ray trees: the camera rays' nodes, then their
    // sets' subtrees as separate items, then the pixels' colours
    const int64_t per_pixel = 2 * (int64_t)std::max(smp.diffuse_samples, 1);   // items a pixel can hand out
    const bool split = smp.stream == RT_STREAM_PIXEL && tree && (int64_t)npix * per_pixel < ((int64_t)1 << 31);
    if (split) {
        RT_CUDA_S(S.root_c.reserve(npix * sizeof(float4)), "node allocation");
        RT_CUDA_S(S.root_sets.reserve(npix * sizeof(int4)), "node allocation");
        RT_CUDA_S(S.nitems.reserve(2 * sizeof(int32_t)), "item counter allocation");
        // items per list (reflection sets, refraction sets)
        int64_t cap = std::min((int64_t)npix * per_pixel / 2, std::max(S.item_cap, (int64_t)npix * 2));
        int32_t n[2] = {0, 0};
        for (int attempt = 0; attempt < 2; ++attempt) {
            RT_CUDA_S(S.items.reserve(2 * (size_t)cap * sizeof(DistItem)), "item allocation");
            RT_CUDA_S(S.item_c.reserve(2 * (size_t)cap * sizeof(float4)), "item colour allocation");
            RT_CUDA_S(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), st), "counter clear");
            RT_CUDA_S(cudaMemsetAsync(S.nitems.ptr, 0, 2 * sizeof(int32_t), st), "item counter clear");
            k_dist_root<<<grid, kTraceThreads, 0, st>>>(sv, cv, ls, mt, dl, dp, (const int4 *)S.area.ptr, s->d_verts,
                                                        (const float *)S.lut.ptr, (float4 *)S.root_c.ptr,
                                                        (int4 *)S.root_sets.ptr, (DistItem *)S.items.ptr, (int32_t)cap,
                                                        (int32_t *)S.nitems.ptr, ctx->d_counters);
            RT_CUDA_S(cudaGetLastError(), "node launch");
            RT_CUDA_S(cudaMemcpyAsync(n, S.nitems.ptr, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, st),
                      "item count read");
            RT_CUDA_S(cudaStreamSynchronize(st), "synchronize");
            if (n[0] >= 0 && n[1] >= 0 && n[0] <= cap && n[1] <= cap) break;
            if (n[0] < 0 || n[1] < 0 || attempt == 1)
                return sfail(RT_ERR_INTERNAL, "rt_render_distributed: item count out of range");
            const int64_t need = std::max(n[0], n[1]);
            cap = std::min((int64_t)npix * per_pixel / 2, need + need / 8);   // grow to fit and run again
        }
        S.item_cap = cap;
        RT_CUDA_S(cudaMemsetAsync(&ctx->d_counters->work, 0, sizeof(int), st), "work counter clear");
        if (n[0] + n[1] > 0)
            k_dist_sub<<<sub_blocks_per_sm() * ctx->sm_count, kTraceThreads, 0, st>>>(
                sv, cv, ls, mt, dl, dp, (const int4 *)S.area.ptr, s->d_verts, (const float *)S.lut.ptr,
                (const DistItem *)S.items.ptr, n[0], n[1], (int32_t)cap, (float4 *)S.item_c.ptr, ctx->d_counters);
        RT_CUDA_S(cudaGetLastError(), "subtree launch");
        k_dist_combine<<<ctx->sm_count * 8, 256, 0, st>>>(cv, mt, (const float4 *)S.root_c.ptr,
                                                          (const int4 *)S.root_sets.ptr, (const float4 *)S.item_c.ptr,
                                                          n[0], n[1], (int32_t)cap, d_rgb, d_f, ctx->d_counters);
    } else {
        k_dist<true><<<grid, kTraceThreads, 0, st>>>(sv, cv, ls, mt, dl, dp, (const int4 *)S.area.ptr, s->d_verts,
                                                     (const float *)S.lut.ptr, rnd, total,
                                                     (const int64_t *)S.prefix64.ptr, nullptr, d_rgb, d_f,
                                                     ctx->d_counters);
    }
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
    if (stream_end)
        *stream_end = smp.stream == RT_STREAM_REFERENCE ? smp.stream_offset + total : (int64_t)c.drawn;
    return status_to_error(c.status);
}
