// rt_wave.cu -- single-frame render kernels with lane-level ray
// replacement (see rt_wave.cuh): the frame is a one-entry job passed as a
// grid constant.
#include "rt_api_internal.cuh"
#include "rt_wave.cuh"

namespace rtc {
namespace {

template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, RT_WAVE_MIN_BLOCKS) k_render_wave(const __grid_constant__ FrameJob job, Counters *ctr)
{
    __shared__ LaneShade shade_state[kTraceThreads];
    wave_loop<8, COUNT>(&job, nullptr, 1, job.items_end, shade_state[threadIdx.x], ctr);
}

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

FrameJob single_job(const SceneView &sc, const CameraView &cam, const MaterialView &mat, uint8_t *rgb, int32_t *ids)
{
    FrameJob J;
    memset(&J, 0, sizeof(J));
    J.sc = sc;
    J.cam = cam;
    J.mat = mat;
    J.rgb = rgb;
    J.ids = ids;
    int tx;
    J.items_begin = 0;
    J.items_end = tiles_of<8>(cam.xres, cam.yres, tx) * 32;
    J.tiles_x = tx;
    return J;
}

}  // namespace

void launch_render_wave(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialView &mat,
                        uint8_t *rgb, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st, bool count)
{
    static const int per_sm = blocks_per_sm(k_render_wave<false>);
    const int grid = per_sm * sm_count;
    FrameJob J = single_job(sc, cam, mat, rgb, ids);
    J.mode = RT_JOB_SHADOW;
    J.nlights = lights.n;
    J.fast_pow = lights.fast_pow;
    for (int i = 0; i < lights.n; ++i) J.lights[i] = lights.l[i];
    if (count)
        k_render_wave<true><<<grid, kTraceThreads, 0, st>>>(J, ctr);
    else
        k_render_wave<false><<<grid, kTraceThreads, 0, st>>>(J, ctr);
}

void launch_render_ao_wave(const SceneView &sc, const CameraView &cam, const MaterialView &mat, int32_t samples,
                           float ao_dist, uint32_t seed, uint8_t *rgb, int32_t *ids, int32_t *ao_count, Counters *ctr,
                           int sm_count, cudaStream_t st, bool count)
{
    static const int per_sm = blocks_per_sm(k_render_wave<false>);
    const int grid = per_sm * sm_count;
    FrameJob J = single_job(sc, cam, mat, rgb, ids);
    J.mode = RT_JOB_AO;
    J.ao_samples = samples;
    J.ao_dist = ao_dist;
    J.ao_seed = seed;
    J.ao_count = ao_count;
    if (count)
        k_render_wave<true><<<grid, kTraceThreads, 0, st>>>(J, ctr);
    else
        k_render_wave<false><<<grid, kTraceThreads, 0, st>>>(J, ctr);
}

}  // namespace rtc
