// rt_trace.cu -- persistent-warp traversal and the fused render kernels.
//
// Every kernel runs a fixed grid (a multiple of the SM count) whose warps
// claim 32 work items at a time from a device counter, so uneven ray costs
// balance across SMs without a scheduler on the host.
#include "rt_kernels.cuh"
#include "rt_traverse.cuh"

namespace rtc {

namespace {

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

__global__ void __launch_bounds__(kTraceThreads) k_trace_closest(SceneView sc, const rt_ray *__restrict__ rays,
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

__global__ void __launch_bounds__(kTraceThreads) k_trace_any(SceneView sc, const rt_ray *__restrict__ rays, int32_t n,
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

// Pixel of work item `item` in 8x4 tiles (one warp = one tile).
__device__ __forceinline__ void tile_pixel(int item, int tiles_x, int &x, int &y)
{
    const int tile = item >> 5, lane = item & 31;
    x = (tile % tiles_x) * 8 + (lane & 7);
    y = (tile / tiles_x) * 4 + (lane >> 3);
}

namespace {

template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads) k_render(SceneView sc, CameraView cam, LightSet lights,
                                                          MaterialView mat, uint8_t *__restrict__ rgb,
                                                          int32_t *__restrict__ ids, Counters *ctr)
{
    const int tiles_x = (cam.xres + 7) >> 3, tiles_y = (cam.yres + 3) >> 2;
    const int items = tiles_x * tiles_y * 32;
    uint32_t status = 0;
    FetchCount fc;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
        HitRecord h;
        h.id = -1;
        h.t = FLT_MAX;
        RayState r;
        bool occ;
        if (live) {
            r = camera_ray(cam, x, y);
            status |= traverse<false, COUNT>(sc, r.o, r.d, FLT_MAX, h, occ, &fc);
        }
        const bool hit = live && h.t < FLT_MAX;
        uint32_t shadow_rays = 0;
        float3 c = cam.background;
        if (hit) {
            const SurfacePoint sp = surface_at(sc, r, h);
            const float3 start = offset_start(sp.dst, sp.geo);
            const float3 kd = material_kd(mat, sp);
            c = make_float3(0.f, 0.f, 0.f);
            for (int l = 0; l < lights.n; ++l) {
                const LightView &L = lights.l[l];
                float3 ldir;
                float len;
                shadow_ray(L, start, ldir, len);
                HitRecord sh;
                bool blocked;
                status |= traverse<true, COUNT>(sc, start, ldir, len, sh, blocked, &fc);
                ++shadow_rays;
                phong_add(L, mat, kd, sp.sn, r.d, ldir, len, blocked ? 0.0f : 1.0f, c);
            }
            c = xadd3(c, mat.ka);
        }
        if (live) {
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            rgb[3 * pix] = clip8(c.x);
            rgb[3 * pix + 1] = clip8(c.y);
            rgb[3 * pix + 2] = clip8(c.z);
            if (ids) ids[pix] = hit ? h.id : -1;
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, hit);
        warp_add(&ctr->secondary, shadow_rays);
    }
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads) k_render_ao(SceneView sc, CameraView cam, MaterialView mat,
                                                             int32_t samples, float ao_dist, uint32_t seed,
                                                             uint8_t *__restrict__ rgb, int32_t *__restrict__ ids,
                                                             int32_t *__restrict__ ao_count, Counters *ctr)
{
    const int tiles_x = (cam.xres + 7) >> 3, tiles_y = (cam.yres + 3) >> 2;
    const int items = tiles_x * tiles_y * 32;
    uint32_t status = 0;
    FetchCount fc;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32);
        if (base >= items) break;
        int x, y;
        tile_pixel(base + (threadIdx.x & 31), tiles_x, x, y);
        const bool live = (x < cam.xres) && (y < cam.yres);
        HitRecord h;
        h.id = -1;
        h.t = FLT_MAX;
        RayState r;
        bool occ;
        if (live) {
            r = camera_ray(cam, x, y);
            status |= traverse<false, COUNT>(sc, r.o, r.d, FLT_MAX, h, occ, &fc);
        }
        const bool hit = live && h.t < FLT_MAX;
        const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
        float3 c = cam.background;
        int made_it = 0;
        if (hit) {
            const SurfacePoint sp = surface_at(sc, r, h);
            const float3 start = offset_start(sp.dst, sp.geo);
            const AOBasis ob = ao_basis(sp.geo);
            for (int s = 0; s < samples; ++s) {
                const float3 d = ao_direction(ob, (uint32_t)pix, (uint32_t)s, seed);
                HitRecord ah;
                bool blocked;
                status |= traverse<true, COUNT>(sc, start, d, ao_dist, ah, blocked, &fc);
                if (!blocked) ++made_it;
            }
            const float3 kd = material_kd(mat, sp);
            const float frac = xdiv((float)made_it, (float)samples);
            c = xadd3(xmul3(kd, frac), mat.ka);
        }
        if (live) {
            rgb[3 * pix] = clip8(c.x);
            rgb[3 * pix + 1] = clip8(c.y);
            rgb[3 * pix + 2] = clip8(c.z);
            if (ids) ids[pix] = hit ? h.id : -1;
            if (ao_count) ao_count[pix] = made_it;
        }
        warp_count(&ctr->primary, live);
        warp_count(&ctr->hits, hit);
        warp_add(&ctr->secondary, hit ? (uint32_t)samples : 0u);
    }
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

}  // namespace

// Persistent grid: SMs x resident blocks per SM (from the occupancy API).
template <typename K>
static int grid_of(K kernel, int sm_count)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceThreads, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 4;
    }
    return sm_count * per_sm;
}

void launch_trace_closest(const SceneView &sc, const rt_ray *rays, int32_t n, rt_hit *hits, Counters *ctr, int sm_count,
                          cudaStream_t st)
{
    static const int grid = grid_of(k_trace_closest, sm_count);
    k_trace_closest<<<grid, kTraceThreads, 0, st>>>(sc, rays, n, hits, ctr);
}

void launch_trace_any(const SceneView &sc, const rt_ray *rays, int32_t n, uint8_t *occ, Counters *ctr, int sm_count,
                      cudaStream_t st)
{
    static const int grid = grid_of(k_trace_any, sm_count);
    k_trace_any<<<grid, kTraceThreads, 0, st>>>(sc, rays, n, occ, ctr);
}

void launch_render(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialView &mat,
                   uint8_t *rgb, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st, bool count)
{
    static const int grid = grid_of(k_render<false>, sm_count);
    if (count)
        k_render<true><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, rgb, ids, ctr);
    else
        k_render<false><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, rgb, ids, ctr);
}

void launch_render_ao(const SceneView &sc, const CameraView &cam, const MaterialView &mat, int32_t samples,
                      float ao_dist, uint32_t seed, uint8_t *rgb, int32_t *ids, int32_t *ao_count, Counters *ctr,
                      int sm_count, cudaStream_t st, bool count)
{
    static const int grid = grid_of(k_render_ao<false>, sm_count);
    if (count)
        k_render_ao<true><<<grid, kTraceThreads, 0, st>>>(sc, cam, mat, samples, ao_dist, seed, rgb, ids, ao_count, ctr);
    else
        k_render_ao<false><<<grid, kTraceThreads, 0, st>>>(sc, cam, mat, samples, ao_dist, seed, rgb, ids, ao_count, ctr);
}

}  // namespace rtc
