// rt_wave.cu -- the fused render kernel with lane-level ray replacement.
//
// Every lane of a persistent warp runs a small state machine: primary ray ->
// one secondary ray per light (or per AO sample) -> shade and store -> claim
// the next pixel.  All lanes advance one traversal step per loop iteration
// whatever kind of ray they carry, and lanes that finish a pixel refill at
// once (warp ballot + one atomicAdd for all of them), so a tile whose pixels
// miss, hit sky, or need long shadow rays no longer leaves lanes idle until
// its slowest pixel is done.  Per-lane shading state waits in shared memory
// while the lane traces its secondary rays.  The arithmetic of every pixel is
// exactly that of rt_render's single-pass kernel (same helpers).
#include "rt_api_internal.cuh"
#include "rt_shade.cuh"

namespace rtc {
namespace {

constexpr int kModeLights = 0;
constexpr int kModeAO = 1;

struct AOParams {
    int32_t samples;
    float dist;
    uint32_t seed;
};

template <int MODE, bool COUNT>
__global__ void __launch_bounds__(kTraceThreads) k_render_wave(SceneView sc, CameraView cam, LightSet lights,
                                                               MaterialView mat, AOParams ao,
                                                               uint8_t *__restrict__ rgb, int32_t *__restrict__ ids,
                                                               int32_t *__restrict__ ao_count, Counters *ctr)
{
    __shared__ LaneShade shade_state[kTraceThreads];
    LaneShade &S = shade_state[threadIdx.x];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lanes_below = (1u << lane) - 1u;
    int tiles_x;
    const int items = tiles_of<8>(cam.xres, cam.yres, tiles_x) * 32;
    const int nsec = (MODE == kModeAO) ? ao.samples : lights.n;
    uint2 stack[kStackSize];
    Trav T;
    FetchCount fc;
    uint32_t status = 0, n_primary = 0, n_hits = 0, n_secondary = 0;
    int x = 0, y = 0;
    int phase = -1;               // -1 idle, 0 primary, k >= 1 secondary ray k-1
    bool queue_open = true;
    for (;;) {
        // refill idle lanes from the pixel queue (one atomic per warp)
        const bool need = phase < 0 && queue_open;
        const uint32_t needmask = __ballot_sync(0xffffffffu, need);
        if (needmask) {
            const int leader = __ffs(needmask) - 1;
            int base = 0;
            if ((int)lane == leader) base = atomicAdd(&ctr->work, __popc(needmask));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + __popc(needmask) >= items) queue_open = false;
            if (need) {
                const int item = base + __popc(needmask & lanes_below);
                if (item < items) {
                    tile_pixel<8>(item, tiles_x, x, y);
                    if (x < cam.xres && y < cam.yres) {
                        const RayState r = camera_ray(cam, x, y);
                        trav_begin(T, sc, r.o, r.d, FLT_MAX, false);
                        phase = 0;
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, phase >= 0)) {
            if (!queue_open) break;
            continue;
        }
        if (phase < 0) continue;
        // one traversal step of whatever ray this lane carries
        if (!trav_step<COUNT>(T, stack, sc, phase > 0, status, &fc)) continue;
        bool done = false;
        if (phase == 0) {
            ++n_primary;
            S.c = cam.background;
            S.id = -1;
            S.made = 0;
            if (T.hit.t < FLT_MAX) {
                ++n_hits;
                RayState r;
                r.o = T.o;
                r.d = T.d;
                const SurfacePoint sp = surface_at(sc, r, T.hit);
                S.id = T.hit.id - sc.tri_base;
                S.kd = material_kd(mat, sp);
                S.sn = sp.sn;
                S.geo = sp.geo;
                S.start = offset_start(sp.dst, sp.geo);
                S.vd = T.d;
                S.c = make_float3(0.f, 0.f, 0.f);
                if (nsec > 0) {
                    phase = 1;
                } else {
                    S.c = xadd3(S.c, mat.ka);
                    done = true;
                }
            } else {
                done = true;
            }
        } else {
            ++n_secondary;
            const int k = phase - 1;
            if (MODE == kModeAO) {
                if (!T.occluded) ++S.made;
            } else {
                float3 ldir;
                float len;
                shadow_ray(lights.l[k], S.start, ldir, len);
                float3 c = S.c;
                phong_add(lights.l[k], mat, S.kd, S.sn, S.vd, ldir, len, T.occluded ? 0.0f : 1.0f, c);
                S.c = c;
            }
            if (phase < nsec) {
                ++phase;
            } else {
                if (MODE == kModeAO) {
                    const float frac = xdiv((float)S.made, (float)nsec);
                    S.c = xadd3(xmul3(S.kd, frac), mat.ka);
                } else {
                    S.c = xadd3(S.c, mat.ka);
                }
                done = true;
            }
        }
        if (!done) {
            // start secondary ray phase-1
            const int k = phase - 1;
            if (MODE == kModeAO) {
                const AOBasis ob = ao_basis(S.geo);
                const uint32_t pix = (uint32_t)x + (uint32_t)y * (uint32_t)cam.xres;
                const float3 d = ao_direction(ob, pix, (uint32_t)k, ao.seed);
                trav_begin(T, sc, S.start, d, ao.dist, true);
            } else {
                float3 ldir;
                float len;
                shadow_ray(lights.l[k], S.start, ldir, len);
                trav_begin(T, sc, S.start, ldir, len, true);
            }
        } else {
            const size_t pix = (size_t)x + (size_t)y * (size_t)cam.xres;
            store_rgb(rgb, pix, S.c);
            if (ids) ids[pix] = S.id;
            if (MODE == kModeAO && ao_count) ao_count[pix] = S.made;
            phase = -1;
        }
    }
    warp_add(&ctr->primary, n_primary);
    warp_add(&ctr->hits, n_hits);
    warp_add(&ctr->secondary, n_secondary);
    if (COUNT) {
        atomicAdd(&ctr->nodes, (unsigned long long)fc.nodes);
        atomicAdd(&ctr->tris, (unsigned long long)fc.tris);
    }
    if (status) atomicOr(&ctr->status, status);
}

template <typename K>
int grid_of(K kernel, int sm_count)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceThreads, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 4;
    }
    return sm_count * per_sm;
}

}  // namespace

void launch_render_wave(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialView &mat,
                        uint8_t *rgb, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st, bool count)
{
    static const int grid = grid_of(k_render_wave<kModeLights, false>, sm_count);
    const AOParams ao{0, 0.f, 0u};
    if (count)
        k_render_wave<kModeLights, true><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, ao, rgb, ids, nullptr, ctr);
    else
        k_render_wave<kModeLights, false><<<grid, kTraceThreads, 0, st>>>(sc, cam, lights, mat, ao, rgb, ids, nullptr, ctr);
}

void launch_render_ao_wave(const SceneView &sc, const CameraView &cam, const MaterialView &mat, int32_t samples,
                           float ao_dist, uint32_t seed, uint8_t *rgb, int32_t *ids, int32_t *ao_count, Counters *ctr,
                           int sm_count, cudaStream_t st, bool count)
{
    static const int grid = grid_of(k_render_wave<kModeAO, false>, sm_count);
    LightSet none;
    none.n = 0;
    const AOParams ao{samples, ao_dist, seed};
    if (count)
        k_render_wave<kModeAO, true><<<grid, kTraceThreads, 0, st>>>(sc, cam, none, mat, ao, rgb, ids, ao_count, ctr);
    else
        k_render_wave<kModeAO, false><<<grid, kTraceThreads, 0, st>>>(sc, cam, none, mat, ao, rgb, ids, ao_count, ctr);
}

}  // namespace rtc
