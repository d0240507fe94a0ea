// rt_trace.cu -- persistent-warp traversal and the fused render kernels.
//
// Every kernel runs a fixed grid (a multiple of the SM count) whose warps
// claim 32 work items at a time from a device counter, so uneven ray costs
// balance across SMs without a scheduler on the host.
#include "rt_shade.cuh"

namespace rtc {

namespace {

__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_trace_closest(SceneView sc, const rt_ray *__restrict__ rays,
                                                                 int32_t n, rt_hit *__restrict__ hits,
                                                                 Counters *ctr)
{
    uint32_t status = 0;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= n) break;
        const int i = base + (threadIdx.x & 31);
        if (i < n) {
            const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
            const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
            HitRecord h;
            bool occ;
            status |= traverse<false>(sc, make_float3(r0.x, r0.y, r0.z), make_float3(r1.x, r1.y, r1.z), FLT_MAX, h, occ);
            reinterpret_cast<float4 *>(hits)[i] = make_float4(__int_as_float(h.id), h.t, h.u, h.v);
        }
    }
    if (status) atomicOr(&ctr->status, status);
}

__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_trace_any(SceneView sc, const rt_ray *__restrict__ rays, int32_t n,
                                                             uint8_t *__restrict__ occluded, Counters *ctr)
{
    uint32_t status = 0;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= n) break;
        const int i = base + (threadIdx.x & 31);
        if (i < n) {
            const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
            const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
            HitRecord h;
            bool occ;
            status |= traverse<true>(sc, make_float3(r0.x, r0.y, r0.z), make_float3(r1.x, r1.y, r1.z), r0.w, h, occ);
            occluded[i] = occ ? 1 : 0;
        }
    }
    if (status) atomicOr(&ctr->status, status);
}

}  // namespace

namespace {

template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_render(SceneView sc, CameraView cam, LightSet lights,
                                                          MaterialView mat, uint8_t *__restrict__ rgb,
                                                          int32_t *__restrict__ ids, Counters *ctr)
{
    int tiles_x;
    const int items = tiles_of<8>(cam.xres, cam.yres, tiles_x) * 32;
    uint32_t status = 0;
    FetchCount fc;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel<8>(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
        PixelOut po;
        po.hit = false;
        po.secondary = 0;
        if (live) {
            po = shade_pixel_lights<COUNT>(sc, cam, lights.l, lights.n, mat, x, y, status, &fc, lights.fast_pow != 0);
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            store_rgb(rgb, pix, po.c);
            if (ids) ids[pix] = po.id;
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, po.hit);
        warp_add(&ctr->secondary, po.secondary);
    }
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

// The unclipped colour (3 floats per pixel, exact specular power) of a
// frame without secondary rays, for the tone-mapping epilogue: the fused
// primary + shadow kernel, its material per triangle from `table` (entry 0
// when the scene has no indices).
template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_render_float(SceneView sc, CameraView cam, LightSet lights,
                                                          MaterialTable table, float *__restrict__ fimg,
                                                          Counters *ctr)
{
    int tiles_x;
    const int items = tiles_of<8>(cam.xres, cam.yres, tiles_x) * 32;
    uint32_t status = 0;
    FetchCount fc;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel<8>(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
        PixelOut po;
        po.hit = false;
        po.secondary = 0;
        if (live) {
            po = shade_pixel_lights<COUNT, true>(sc, cam, lights.l, lights.n, table.m[0], x, y, status, &fc, false,
                                                 &table);
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            fimg[3 * pix] = po.c.x;
            fimg[3 * pix + 1] = po.c.y;
            fimg[3 * pix + 2] = po.c.z;
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, po.hit);
        warp_add(&ctr->secondary, po.secondary);
    }
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

// k_render with the hit triangle's material taken from a table
// (rt_render_materials without mirror or refracted rays): a separate kernel
// so that the single-material one keeps its code and parameter block.
template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_render_table(SceneView sc, CameraView cam, LightSet lights,
                                                          MaterialView mat, uint8_t *__restrict__ rgb,
                                                          int32_t *__restrict__ ids, Counters *ctr,
                                                          MaterialTable table)
{
    int tiles_x;
    const int items = tiles_of<8>(cam.xres, cam.yres, tiles_x) * 32;
    uint32_t status = 0;
    FetchCount fc;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel<8>(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
        PixelOut po;
        po.hit = false;
        po.secondary = 0;
        if (live) {
            po = shade_pixel_lights<COUNT, true>(sc, cam, lights.l, lights.n, mat, x, y, status, &fc,
                                                 lights.fast_pow != 0, &table);
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            store_rgb(rgb, pix, po.c);
            if (ids) ids[pix] = po.id;
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, po.hit);
        warp_add(&ctr->secondary, po.secondary);
    }
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

// RT_AO_SPREAD: spread each warp's AO rays over all its lanes (default), or
// one pixel's rays per lane.
#ifndef RT_AO_SPREAD
#define RT_AO_SPREAD 1
#endif

template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_render_ao(SceneView sc, CameraView cam, MaterialView mat,
                                                             int32_t samples, float ao_dist, uint32_t seed,
                                                             uint8_t *__restrict__ rgb, int32_t *__restrict__ ids,
                                                             int32_t *__restrict__ ao_count, Counters *ctr)
{
    int tiles_x;
    const int items = tiles_of<8>(cam.xres, cam.yres, tiles_x) * 32;
    uint32_t status = 0;
    FetchCount fc;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel<8>(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
#if RT_AO_SPREAD
        // primary ray per lane; then the warp's hits * samples AO rays are
        // spread over all 32 lanes (a lane whose pixel missed takes rays of
        // its neighbours), each ray's origin and basis fetched from the lane
        // that owns its pixel, the unoccluded counts gathered per owner in
        // shared memory.  Same rays, same counts as shade_pixel_ao.
        __shared__ int made_s[kTraceThreads];
        const int lane = threadIdx.x & 31;
        const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
        bool hit = false;
        int32_t id = -1;
        float3 start = make_float3(0.f, 0.f, 0.f), kd = make_float3(0.f, 0.f, 0.f);
        AOBasis ob;
        ob.T = ob.B = ob.g = make_float3(0.f, 0.f, 0.f);
        if (live) {
            const RayState r = camera_ray(cam, x, y);
            HitRecord h;
            bool occ;
            status |= traverse<false, COUNT>(sc, r.o, r.d, FLT_MAX, h, occ, &fc);
            hit = h.t < FLT_MAX;
            if (hit) {
                id = h.id - sc.tri_base;
                const SurfacePoint sp = surface_at(sc, r, h);
                start = offset_start(sp.dst, sp.geo);
                ob = ao_basis(sp.geo);
                kd = material_kd(mat, sp);
            }
        }
        made_s[threadIdx.x] = 0;
        __syncwarp();
        const uint32_t hitmask = __ballot_sync(0xffffffffu, hit);
        const int total = __popc(hitmask) * samples;
        for (int r0 = 0; r0 < total; r0 += 32) {
            const int r = r0 + lane;
            const bool active = r < total;
            const int q = active ? r / samples : 0;
            const int k = active ? r - q * samples : 0;
            const int owner = active ? (int)__fns(hitmask, 0, q + 1) : lane;
            const float3 o = make_float3(__shfl_sync(0xffffffffu, start.x, owner),
                                         __shfl_sync(0xffffffffu, start.y, owner),
                                         __shfl_sync(0xffffffffu, start.z, owner));
            AOBasis b;
            b.T = make_float3(__shfl_sync(0xffffffffu, ob.T.x, owner), __shfl_sync(0xffffffffu, ob.T.y, owner),
                              __shfl_sync(0xffffffffu, ob.T.z, owner));
            b.B = make_float3(__shfl_sync(0xffffffffu, ob.B.x, owner), __shfl_sync(0xffffffffu, ob.B.y, owner),
                              __shfl_sync(0xffffffffu, ob.B.z, owner));
            b.g = make_float3(__shfl_sync(0xffffffffu, ob.g.x, owner), __shfl_sync(0xffffffffu, ob.g.y, owner),
                              __shfl_sync(0xffffffffu, ob.g.z, owner));
            const uint32_t opix = (uint32_t)__shfl_sync(0xffffffffu, (int)pix, owner);
            if (active) {
                const float3 d = ao_direction(b, opix, (uint32_t)k, seed);
                HitRecord ah;
                bool blocked;
                status |= traverse<true, COUNT>(sc, o, d, ao_dist, ah, blocked, &fc);
                if (!blocked) atomicAdd(&made_s[(threadIdx.x & ~31) + owner], 1);
            }
        }
        __syncwarp();
        if (live) {
            float3 c = cam.background;
            int made = 0;
            if (hit) {
                made = made_s[threadIdx.x];
                const float frac = xdiv((float)made, (float)samples);
                c = xadd3(xmul3(kd, frac), mat.ka);
            }
            store_rgb(rgb, pix, c);
            if (ids) ids[pix] = id;
            if (ao_count) ao_count[pix] = made;
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, hit);
        warp_add(&ctr->secondary, hit ? (uint32_t)samples : 0u);
#else
        PixelOut po;
        po.hit = false;
        po.secondary = 0;
        if (live) {
            po = shade_pixel_ao<COUNT>(sc, cam, mat, samples, ao_dist, seed, x, y, status, &fc);
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            store_rgb(rgb, pix, po.c);
            if (ids) ids[pix] = po.id;
            if (ao_count) ao_count[pix] = po.ao_made;
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, po.hit);
        warp_add(&ctr->secondary, po.secondary);
#endif
    }
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

// Anti-aliased frame (camera x_a_res / y_a_res, camera.h:55-62, averaged by
// clip_image_to_rgb, camera.h:289-319): one output pixel per lane; its
// aa_x * aa_y samples on the supersampled camera grid are shaded and summed
// a_x outer, a_y inner, divided by their count, clamped and truncated.  With
// the single-precision specular power, a pixel whose average lands within
// the truncation guard of an integer is queued (redo) for k_render_aa_fix,
// which recomputes it from samples shaded with the exact power in a compact
// second pass, so that no warp waits on one lane's exact re-shade.
template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_render_aa(SceneView sc, CameraView cam,
                                                             LightSet lights, MaterialView mat, int32_t aa_x,
                                                             int32_t aa_y, int32_t out_x, int32_t out_y,
                                                             uint8_t *__restrict__ rgb, int32_t *__restrict__ redo,
                                                             Counters *ctr)
{
    const int S = aa_x * aa_y;
    const float nsamples = (float)S;
    uint32_t status = 0;
    FetchCount fc;
    int tiles_x;
    const int items = tiles_of<8>(out_x, out_y, tiles_x) * 32;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel<8>(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < out_x) && (y < out_y);
        uint32_t primary = 0, hits = 0, secondary = 0;
        if (live) {
            float3 sum = make_float3(0.f, 0.f, 0.f);
            for (int ax = 0; ax < aa_x; ++ax)
                for (int ay = 0; ay < aa_y; ++ay) {
                    const PixelOut po = shade_pixel_lights<COUNT>(sc, cam, lights.l, lights.n, mat, x * aa_x + ax,
                                                                  y * aa_y + ay, status, &fc, lights.fast_pow != 0);
                    sum = xadd3(sum, po.c);
                    ++primary;
                    hits += po.hit ? 1u : 0u;
                    secondary += po.secondary;
                }
            const float3 avg = make_float3(xdiv(sum.x, nsamples), xdiv(sum.y, nsamples), xdiv(sum.z, nsamples));
            const int32_t pix = x + y * out_x;
            if (lights.fast_pow && near_truncation(avg)) {
                const int slot = atomicAdd(&ctr->redo, 1);
                if (slot < out_x * out_y) redo[slot] = pix;
            } else {
                store_rgb(rgb, (size_t)pix, avg);
            }
        }
        warp_add(&ctr->primary, primary);
        warp_add(&ctr->hits, hits);
        warp_add(&ctr->secondary, secondary);
    }
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

// k_render_aa with one sample per lane (aa_x * aa_y <= 32): a warp covers
// a tile of output pixels, lane g * S + s taking sample s (x outer, y
// inner) of pixel g; the pixel's first lane sums the samples in that order
// (shuffled from their lanes), so the frame is the per-pixel loop's bit for
// bit, while the warp's lanes trace one sample each instead of looping
// over a pixel's samples.
template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_render_aa_lanes(SceneView sc, CameraView cam,
                                                             LightSet lights, MaterialView mat, int32_t aa_x,
                                                             int32_t aa_y, int32_t out_x, int32_t out_y,
                                                             uint8_t *__restrict__ rgb, int32_t *__restrict__ redo,
                                                             Counters *ctr)
{
    const int S = aa_x * aa_y;
    const float nsamples = (float)S;
    uint32_t status = 0;
    FetchCount fc;
    // one sample per lane: a warp covers a tile of tw x th output
    // pixels, lane g * S + s taking sample s (x outer, y inner) of
    // pixel g; the pixel's first lane sums the samples in that order
    const int per = 32 / S;
    const int tw = per >= 8 ? 4 : per, th = per >= 8 ? per / 4 : 1;
    const int lane = threadIdx.x & 31;
    const int g = lane / S, smp = lane % S;
    const int ax = smp / aa_y, ay = smp % aa_y;
    const int tiles_x = (out_x + tw - 1) / tw;
    const int ntiles = tiles_x * ((out_y + th - 1) / th);
    for (;;) {
        const int tile = warp_claim(&ctr->work, 32) >> 5;
        if (tile >= ntiles) break;
        const int x = (tile % tiles_x) * tw + g % tw, y = (tile / tiles_x) * th + g / tw;
        const bool live = g < tw * th && x < out_x && y < out_y;
        PixelOut po;
        po.c = make_float3(0.f, 0.f, 0.f);
        po.hit = false;
        po.secondary = 0;
        if (live)
            po = shade_pixel_lights<COUNT>(sc, cam, lights.l, lights.n, mat, x * aa_x + ax, y * aa_y + ay, status,
                                           &fc, lights.fast_pow != 0);
        const int first = g * S;
        float3 sum = make_float3(0.f, 0.f, 0.f);
        for (int k = 0; k < S; ++k) {
            const int src = min(first + k, 31);
            const float3 q = make_float3(__shfl_sync(0xffffffffu, po.c.x, src), __shfl_sync(0xffffffffu, po.c.y, src),
                                         __shfl_sync(0xffffffffu, po.c.z, src));
            sum = xadd3(sum, q);
        }
        if (live && smp == 0) {
            const float3 avg = make_float3(xdiv(sum.x, nsamples), xdiv(sum.y, nsamples), xdiv(sum.z, nsamples));
            const int32_t pix = x + y * out_x;
            if (lights.fast_pow && near_truncation(avg)) {
                const int slot = atomicAdd(&ctr->redo, 1);
                if (slot < out_x * out_y) redo[slot] = pix;
            } else {
                store_rgb(rgb, (size_t)pix, avg);
            }
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, po.hit);
        warp_add(&ctr->secondary, po.secondary);
    }
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

// The queued pixels of k_render_aa, one per thread, every sample shaded
// with the exact specular power.
__global__ void __launch_bounds__(kTraceThreads, RT_RENDER_MIN_BLOCKS) k_render_aa_fix(SceneView sc, CameraView cam,
                                                                 LightSet lights, MaterialView mat, int32_t aa_x,
                                                                 int32_t aa_y, int32_t out_x,
                                                                 uint8_t *__restrict__ rgb,
                                                                 const int32_t *__restrict__ redo, Counters *ctr)
{
    const int32_t n = min(ctr->redo, out_x * (cam.yres / aa_y));
    const float nsamples = (float)(aa_x * aa_y);
    uint32_t status = 0;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t pix = redo[i];
        const int x = pix % out_x, y = pix / out_x;
        float3 sum = make_float3(0.f, 0.f, 0.f);
        for (int ax = 0; ax < aa_x; ++ax)
            for (int ay = 0; ay < aa_y; ++ay) {
                const PixelOut po = shade_pixel_lights<false>(sc, cam, lights.l, lights.n, mat, x * aa_x + ax,
                                                              y * aa_y + ay, status, nullptr, false);
                sum = xadd3(sum, po.c);
            }
        store_rgb(rgb, (size_t)pix,
                  make_float3(xdiv(sum.x, nsamples), xdiv(sum.y, nsamples), xdiv(sum.z, nsamples)));
    }
    if (status) atomicOr(&ctr->status, status);
}

// Frame with secondary rays or per-triangle materials: one pixel per lane,
// the pixel's ray tree walked by shade_pixel_tree (its pending rays in a
// per-thread frame stack).  fimg non-null: the unclipped colour (3 floats
// per pixel) is written instead of RGB8.
// Resident blocks per SM the ray-tree kernel is compiled for (its frame
// stack lives in local memory either way).  Measured on the glass-sphere
// frame (512^2, 41k triangles): 1 / 4 / 5 / 6 / 8 blocks (142 / 128 / 96 /
// 80 / 64 registers) give 0.83 / 0.77 / 0.73 / 0.75 / 0.85 ms.
#ifndef RT_TREE_MIN_BLOCKS
#define RT_TREE_MIN_BLOCKS 5
#endif

template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, RT_TREE_MIN_BLOCKS) k_render_tree(SceneView sc, CameraView cam, LightSet lights,
                                                               MaterialTable mt, uint8_t *__restrict__ rgb,
                                                               float *__restrict__ fimg, int32_t *__restrict__ ids,
                                                               Counters *ctr)
{
    TreeFrame frames[RT_MAX_BOUNCES + 1];
    int tiles_x;
    const int items = tiles_of<8>(cam.xres, cam.yres, tiles_x) * 32;
    uint32_t status = 0;
    FetchCount fc;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel<8>(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
        PixelOut po;
        po.hit = false;
        po.secondary = 0;
        if (live) {
            po = shade_pixel_tree<COUNT>(sc, cam, lights.l, lights.n, mt, x, y, frames, status, &fc);
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            if (fimg) {
                fimg[3 * pix] = po.c.x;
                fimg[3 * pix + 1] = po.c.y;
                fimg[3 * pix + 2] = po.c.z;
            } else {
                store_rgb(rgb, pix, po.c);
            }
            if (ids) ids[pix] = po.id;
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, po.hit);
        warp_add(&ctr->secondary, po.secondary);
    }
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

// Smallest and largest of n indices (out[0], out[1]; n >= 0).
__global__ void k_index_range(const int32_t *__restrict__ v, int32_t n, int32_t *out)
{
    int32_t lo = 0, hi = 0;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t x = v[i];
        lo = min(lo, x);
        hi = max(hi, x);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&out[0], lo);
        atomicMax(&out[1], hi);
    }
}

}  // namespace

// Persistent grid: the context's SMs x resident blocks per SM.  The
// occupancy is a property of the kernel alone, so each launcher asks the
// occupancy API once and scales it by the SM count of the calling context.
template <typename K>
static int blocks_per_sm(K kernel)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceThreads, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 4;
    }
    return per_sm;
}

void launch_trace_closest(const SceneView &sc, const rt_ray *rays, int32_t n, rt_hit *hits, Counters *ctr, int sm_count,
                          cudaStream_t st)
{
    static const int per_sm = blocks_per_sm(k_trace_closest);
    const int grid = per_sm * sm_count;
    k_trace_closest<<<grid, kTraceThreads, 0, st>>>(sc, rays, n, hits, ctr);
}

void launch_trace_any(const SceneView &sc, const rt_ray *rays, int32_t n, uint8_t *occ, Counters *ctr, int sm_count,
                      cudaStream_t st)
{
    static const int per_sm = blocks_per_sm(k_trace_any);
    const int grid = per_sm * sm_count;
    k_trace_any<<<grid, kTraceThreads, 0, st>>>(sc, rays, n, occ, ctr);
}

void launch_render(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialView &mat,
                   uint8_t *rgb, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st, bool count)
{
    static const int per_sm = blocks_per_sm(k_render<false>);
    const int grid = per_sm * sm_count;
    if (count)
        k_render<true><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, rgb, ids, ctr);
    else
        k_render<false><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, rgb, ids, ctr);
}

void launch_render_float(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialTable &mt,
                         float *fimg, Counters *ctr, int sm_count, cudaStream_t st, bool count)
{
    static const int per_sm = blocks_per_sm(k_render_float<false>);
    const int grid = per_sm * sm_count;
    if (count)
        k_render_float<true><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mt, fimg, ctr);
    else
        k_render_float<false><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mt, fimg, ctr);
}

void launch_render_table(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialTable &mt,
                         uint8_t *rgb, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st, bool count)
{
    static const int per_sm = blocks_per_sm(k_render_table<false>);
    const int grid = per_sm * sm_count;
    if (count)
        k_render_table<true><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mt.m[0], rgb, ids, ctr, mt);
    else
        k_render_table<false><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mt.m[0], rgb, ids, ctr, mt);
}

void launch_render_tree(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialTable &mt,
                        uint8_t *rgb, float *fimg, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st,
                        bool count)
{
    static const int per_sm = blocks_per_sm(k_render_tree<false>);
    const int grid = per_sm * sm_count;
    if (count)
        k_render_tree<true><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mt, rgb, fimg, ids, ctr);
    else
        k_render_tree<false><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mt, rgb, fimg, ids, ctr);
}

void launch_index_range(const int32_t *v, int32_t n, int32_t *out, cudaStream_t st)
{
    cudaMemsetAsync(out, 0, 2 * sizeof(int32_t), st);
    const int blocks = (n + 255) / 256;
    const int grid = blocks < 1 ? 1 : (blocks > 1216 ? 1216 : blocks);
    k_index_range<<<grid, 256, 0, st>>>(v, n, out);
}

void launch_render_aa(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialView &mat,
                      int32_t aa_x, int32_t aa_y, int32_t out_x, int32_t out_y, uint8_t *rgb, int32_t *redo,
                      Counters *ctr, int sm_count, cudaStream_t st, bool count)
{
    static const int per_sm = blocks_per_sm(k_render_aa<false>);
    const int grid = per_sm * sm_count;
    if (aa_x * aa_y <= 32) {
        if (count)
            k_render_aa_lanes<true><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, aa_x, aa_y, out_x, out_y,
                                                                     rgb, redo, ctr);
        else
            k_render_aa_lanes<false><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, aa_x, aa_y, out_x, out_y,
                                                                      rgb, redo, ctr);
    } else if (count)
        k_render_aa<true><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, aa_x, aa_y, out_x, out_y, rgb, redo,
                                                           ctr);
    else
        k_render_aa<false><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, aa_x, aa_y, out_x, out_y, rgb, redo,
                                                            ctr);
    if (lights.fast_pow)
        k_render_aa_fix<<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, aa_x, aa_y, out_x, rgb, redo, ctr);
}

void launch_render_ao(const SceneView &sc, const CameraView &cam, const MaterialView &mat, int32_t samples,
                      float ao_dist, uint32_t seed, uint8_t *rgb, int32_t *ids, int32_t *ao_count, Counters *ctr,
                      int sm_count, cudaStream_t st, bool count)
{
    static const int per_sm = blocks_per_sm(k_render_ao<false>);
    const int grid = per_sm * sm_count;
    if (count)
        k_render_ao<true><<<grid, kTraceThreads, 0, st>>>(sc, cam, mat, samples, ao_dist, seed, rgb, ids, ao_count, ctr);
    else
        k_render_ao<false><<<grid, kTraceThreads, 0, st>>>(sc, cam, mat, samples, ao_dist, seed, rgb, ids, ao_count, ctr);
}

}  // namespace rtc
