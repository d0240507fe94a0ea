// rt_wave.cuh -- the lane-replacement render loop shared by the
// single-frame and batched kernels.
//
// Each lane carries one pixel through a small state machine:
//   IDLE -> (claim a pixel) -> TRAVERSE primary -> FINISHED -> (shade / set
//   up the next shadow or AO ray) -> TRAVERSE ... -> FINISHED -> (store) ->
//   IDLE.
// A loop iteration does ONE kind of work for the whole warp: if at least
// kWaveBatch lanes wait in FINISHED (or no lane is traversing) they all take
// their transition together; if at least kWaveBatch lanes are IDLE (or none
// is traversing) they all claim pixels together (one atomicAdd); otherwise
// every TRAVERSE lane advances one traversal step.  Shading and ray set-up
// therefore run with most lanes active, while traversal keeps lanes busy
// across pixels of different cost.  Per-lane shading state waits in shared
// memory.  Pixel arithmetic is that of the single-pass kernels.
#pragma once

#include "rt_shade.cuh"

namespace rtc {

constexpr int kWaveBatch = 16;

// One frame of work: a scene, a camera, lights or AO, outputs, and the range
// of work items (32-pixel tiles) it owns in the queue.
struct FrameJob {
    SceneView sc;
    CameraView cam;
    MaterialView mat;
    LightView lights[RT_MAX_LIGHTS];
    int32_t nlights;
    int32_t fast_pow;
    int32_t mode;              // RT_JOB_SHADOW or RT_JOB_AO
    int32_t ao_samples;
    float ao_dist;
    uint32_t ao_seed;
    int32_t tiles_x;
    int32_t items_begin;
    int32_t items_end;
    uint8_t *rgb;
    int32_t *ids;
    int32_t *ao_count;
};

enum : int { kLaneIdle = 0, kLaneTraverse = 1, kLaneFinished = 2 };

// Jobs: `single` (nullable) is the one job of a single-frame launch; else
// the table `jobs` of njobs entries is searched by item.
template <int TW, bool COUNT>
__device__ __forceinline__ void wave_loop(const FrameJob *single, const FrameJob *__restrict__ jobs, int32_t njobs,
                                          int32_t total_items, LaneShade &S, Counters *ctr)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lanes_below = (1u << lane) - 1u;
    uint2 stack[kStackSize];
    Trav T;
    FetchCount fc;
    uint32_t status = 0, n_primary = 0, n_hits = 0, n_secondary = 0;
    int x = 0, y = 0, j = 0;
    int state = kLaneIdle;
    int phase = 0;            // 0 primary, k >= 1 secondary ray k-1
    bool queue_open = true;
    for (;;) {
        const uint32_t trav = __ballot_sync(0xffffffffu, state == kLaneTraverse);
        const uint32_t fin = __ballot_sync(0xffffffffu, state == kLaneFinished);
        const uint32_t idle = ~(trav | fin);
        if (fin && (__popc(fin) >= kWaveBatch || !trav)) {
            // ---- transitions of every finished lane, together
            if (state == kLaneFinished) {
                const FrameJob &J = single ? *single : jobs[j];
                const bool ao = J.mode == RT_JOB_AO;
                const int nsec = ao ? J.ao_samples : J.nlights;
                bool done = false;
                if (phase == 0) {
                    ++n_primary;
                    S.c = J.cam.background;
                    S.id = -1;
                    S.made = 0;
                    if (T.hit.t < FLT_MAX) {
                        ++n_hits;
                        RayState r;
                        r.o = T.o;
                        r.d = T.d;
                        const SurfacePoint sp = surface_at(J.sc, r, T.hit);
                        S.id = T.hit.id - J.sc.tri_base;
                        S.kd = material_kd(J.mat, sp);
                        S.sn = sp.sn;
                        S.geo = sp.geo;
                        S.start = offset_start(sp.dst, sp.geo);
                        S.vd = T.d;
                        S.c = make_float3(0.f, 0.f, 0.f);
                        if (nsec > 0) phase = 1;
                        else { S.c = xadd3(S.c, J.mat.ka); done = true; }
                    } else {
                        done = true;
                    }
                } else {
                    ++n_secondary;
                    const int k = phase - 1;
                    if (ao) {
                        if (!T.occluded) ++S.made;
                    } else {
                        float3 ldir;
                        float len;
                        shadow_ray(J.lights[k], S.start, ldir, len);
                        float3 c = S.c;
                        const float magn = T.occluded ? 0.0f : 1.0f;
                        if (T.occluded) S.made |= 1 << k;
                        if (J.fast_pow) phong_add<false>(J.lights[k], J.mat, S.kd, S.sn, S.vd, ldir, len, magn, c);
                        else phong_add<true>(J.lights[k], J.mat, S.kd, S.sn, S.vd, ldir, len, magn, c);
                        S.c = c;
                    }
                    if (phase < nsec) {
                        ++phase;
                    } else {
                        if (ao) {
                            S.c = xadd3(xmul3(S.kd, xdiv((float)S.made, (float)nsec)), J.mat.ka);
                        } else {
                            S.c = xadd3(S.c, J.mat.ka);
                            if (J.fast_pow && near_truncation(S.c))
                                S.c = shade_lights_exact(J.lights, nsec, J.mat, S.kd, S.sn, S.vd, S.start,
                                                         (uint32_t)S.made);
                        }
                        done = true;
                    }
                }
                if (!done) {
                    const int k = phase - 1;
                    if (ao) {
                        const AOBasis ob = ao_basis(S.geo);
                        const uint32_t pix = (uint32_t)x + (uint32_t)y * (uint32_t)J.cam.xres;
                        trav_begin(T, J.sc, S.start, ao_direction(ob, pix, (uint32_t)k, J.ao_seed), J.ao_dist, true);
                    } else {
                        float3 ldir;
                        float len;
                        shadow_ray(J.lights[k], S.start, ldir, len);
                        trav_begin(T, J.sc, S.start, ldir, len, true);
                    }
                    state = kLaneTraverse;
                } else {
                    const size_t pix = (size_t)x + (size_t)y * (size_t)J.cam.xres;
                    store_rgb(J.rgb, pix, S.c);
                    if (J.ids) J.ids[pix] = S.id;
                    if (ao && J.ao_count) J.ao_count[pix] = S.made;
                    state = kLaneIdle;
                }
            }
            continue;
        }
        if (queue_open && (__popc(idle) >= kWaveBatch || (!trav && idle))) {
            // ---- every idle lane claims a pixel (one atomic per warp)
            int base = 0;
            if (lane == 0) base = atomicAdd(&ctr->work, __popc(idle));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + __popc(idle) >= total_items) queue_open = false;
            if (state == kLaneIdle) {
                const int item = base + __popc(idle & lanes_below);
                if (item < total_items) {
                    if (!single) {
                        int lo = 0, hi = njobs - 1;
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (__ldg(&jobs[mid].items_begin) <= item) lo = mid; else hi = mid - 1;
                        }
                        j = lo;
                    }
                    const FrameJob &J = single ? *single : jobs[j];
                    tile_pixel<TW>(item - J.items_begin, J.tiles_x, x, y);
                    if (x < J.cam.xres && y < J.cam.yres) {
                        const RayState r = camera_ray(J.cam, x, y);
                        trav_begin(T, J.sc, r.o, r.d, FLT_MAX, false);
                        phase = 0;
                        state = kLaneTraverse;
                    }
                }
            }
            continue;
        }
        if (!trav) {
            if (!queue_open) break;
            continue;
        }
        // ---- one traversal step of every traversing lane
        if (state == kLaneTraverse) {
            const FrameJob &J = single ? *single : jobs[j];
            if (trav_step<COUNT>(T, stack, J.sc, phase > 0, status, &fc)) state = kLaneFinished;
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

}  // namespace rtc
