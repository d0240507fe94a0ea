// rt_api_internal.cuh -- host-side objects behind the C ABI handles.
#pragma once

#include <cmath>
#include <string>

#include "rt_build.cuh"
#include "rt_internal.cuh"
#include "rt_kernels.cuh"

namespace rtc {

// Grow-only device buffer.
struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t bytes);
    void release();
};

bool is_device_ptr(const void *p);
CameraView make_camera_view(const rt_camera &c);
LightView make_light_view(const rt_light &l);
MaterialView make_material_view(const rt_material &m);
rt_status set_error(rt_status code, const char *msg);
rt_status set_cuda_error(cudaError_t e, const char *what);
rt_status status_to_error(uint32_t st);

// Live contexts per device, kept for the allocation-free entry point: its
// cached scratch address on a device is forgotten when the last context on
// that device is destroyed (a device reset in between may move the module).
void noalloc_context_opened(int device);
void noalloc_context_closed(int device);

// Per-context buffers of the soft-shadow path (rt_soft.cu), made on first use.
struct SoftState;
void soft_release(rt_context *ctx);

}  // namespace rtc

struct rt_context {
    int device = 0;
    int sm_count = 1;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    rtc::Counters *d_counters = nullptr;
    rtc::Counters *h_counters = nullptr;   // pinned
    int32_t *h_scratch = nullptr;          // pinned
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    rtc::DevBuf stage_a, stage_b, stage_c;
    rtc::DevBuf redo;                      // pixels queued for an exact second pass
    rtc::DevBuf fimg;                      // float frame of rt_render_tone_mapped
    rtc::DevBuf tone;                      // its tone-mapping accumulators
    bool count_fetches = false;
    int render_kernel = RT_KERNEL_PIXEL;
    int isect = RT_ISECT_REFERENCE;
    int builder = RT_BUILDER_HPLOC;
    int morton_bits = 0;                   // RT_OPT_MORTON_BITS
    rtc::SoftState *soft = nullptr;        // rt_render_soft_shadows state
};

struct rt_scene {
    rt_context *ctx = nullptr;
    int32_t nverts = 0, ntris = 0;
    float *d_verts = nullptr;
    int3 *d_idx = nullptr;
    float *d_vattr = nullptr;
    uint32_t *d_flags = nullptr;
    rtc::ShadeTri *d_shade = nullptr;
    int32_t *d_mat = nullptr;             // material index per triangle (rt_scene_set_materials)
    int32_t mat_max = -1;                 // largest index in d_mat (-1: none set)
    float *d_cnorm = nullptr;             // corner normals, 9 floats per triangle (rt_scene_set_normals)
    rtc::WideNode *d_nodes = nullptr;
    rtc::PackedTri *d_tris = nullptr;
    int32_t nnodes = 0, tri_slots = 0, depth = 0;
    bool built = false;
    rtc::DevBuf temp;
    rtc::RefitArrays refit;   // the last build's tree, for rt_scene_refit_vertices
};

namespace rtc {
SceneView scene_view(const rt_scene *s);
}
