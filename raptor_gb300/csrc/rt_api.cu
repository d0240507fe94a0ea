// rt_api.cu -- the C ABI (include/rtcore.h): contexts, scenes, staging of
// host buffers, and launch of the build / trace / render kernels.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "rt_build.cuh"
#include "rt_kernels.cuh"
#include "rt_api_internal.cuh"

using namespace rtc;

namespace {

thread_local std::string g_last_error;

rt_status fail(rt_status code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

rt_status cuda_fail(cudaError_t e, const char *what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA, m);
}

#define RT_CUDA(call, what)                          \
    do {                                             \
        cudaError_t _e = (call);                     \
        if (_e != cudaSuccess) return cuda_fail(_e, what); \
    } while (0)

// Make the context's device current for the duration of a call.
struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

namespace rtc {

bool is_device_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

cudaError_t DevBuf::reserve(size_t bytes)
{
    if (bytes <= cap) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    const size_t want = bytes + bytes / 4 + 256;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) cap = want;
    return e;
}

void DevBuf::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
}

CameraView make_camera_view(const rt_camera &c)
{
    // base_camera axes pass through the identity quaternion rotation
    // (sdl_wrappers/base_camera.h, common/quaternion_t.h:166-169); restated
    // literally so the signs of zero components match the reference.
    const auto rot = [](const float *p) {
        const float qw = 1.0f, qx = 0.0f, qy = 0.0f, qz = 0.0f;
        const float c1x = (qy * p[2]) - (qz * p[1]), c1y = (qz * p[0]) - (qx * p[2]), c1z = (qx * p[1]) - (qy * p[0]);
        const float c2x = (qy * c1z) - (qz * c1y), c2y = (qz * c1x) - (qx * c1z), c2z = (qx * c1y) - (qy * c1x);
        const float w2 = 2.0f * qw;
        return make_float3((p[0] + (2.0f * c2x)) + (w2 * c1x), (p[1] + (2.0f * c2y)) + (w2 * c1y),
                           (p[2] + (2.0f * c2z)) + (w2 * c1z));
    };
    CameraView v;
    v.c = make_float3(c.pos[0], c.pos[1], c.pos[2]);
    v.X = rot(c.x_axis);
    v.Y = rot(c.y_axis);
    v.Z = rot(c.z_axis);
    v.x_m = -c.w;
    v.y_m = -c.h;
    v.x_inc = (c.w * 2.0f) / (float)c.xres;   // camera.h:60
    v.y_inc = (c.h * 2.0f) / (float)c.yres;
    v.t = c.t;
    v.xres = c.xres;
    v.yres = c.yres;
    v.background = make_float3(c.background[0], c.background[1], c.background[2]);
    return v;
}

LightView make_light_view(const rt_light &l)
{
    LightView v;
    v.kind = l.kind & ~RT_LIGHT_UNIT_RGB;
    if (l.kind & RT_LIGHT_UNIT_RGB)
        v.rgb255 = make_float3(l.rgb[0], l.rgb[1], l.rgb[2]);
    else
        v.rgb255 = make_float3(l.rgb[0] / 255.0f, l.rgb[1] / 255.0f, l.rgb[2] / 255.0f);   // light.h:17-34
    v.pos = make_float3(l.pos[0], l.pos[1], l.pos[2]);
    v.dir = make_float3(l.dir[0], l.dir[1], l.dir[2]);
    v.d = l.d;
    v.s_a = (v.kind == RT_LIGHT_SPOT) ? l.s_a : 0.0f;
    v.s_b = (v.kind == RT_LIGHT_SPOT) ? l.s_b : 0.0f;
    // a spot light without a cone is directional to light::find_rays
    // (light.h:65: n is not the spherical constructor's (2, 2, 2), s_b == 0)
    if (v.kind == RT_LIGHT_SPOT && l.s_b == 0.0f) v.kind = RT_LIGHT_DIRECTIONAL;
    v.radius = 0.0f;
    // light::find_major_direction (light.h:172-219)
    const float nx = l.dir[0], ny = l.dir[1], nz = l.dir[2];
    bool neg;
    if (std::fabs(nx) > std::fabs(ny)) neg = (std::fabs(nx) > std::fabs(nz)) ? (nx < 0.0f) : (nz < 0.0f);
    else neg = (std::fabs(ny) > std::fabs(nz)) ? (ny < 0.0f) : (nz < 0.0f);
    v.dist_sign = neg ? -1.0e15f : 1.0e15f;
    return v;
}

MaterialView make_material_view(const rt_material &m)
{
    MaterialView v;
    v.ka = make_float3(m.ka[0], m.ka[1], m.ka[2]);
    v.kd = make_float3(m.kd[0], m.kd[1], m.kd[2]);
    v.ks = make_float3(m.ks[0], m.ks[1], m.ks[2]);
    v.ns = m.ns;
    v.rf = m.rf;
    v.tran = m.tran;
    v.ri = m.ri;
    v.flags = m.flags;
    return v;
}

SceneView scene_view(const rt_scene *s)
{
    SceneView v;
    v.nodes = s->d_nodes;
    v.tris = s->d_tris;
    v.shade = s->d_shade;
    v.idx = s->d_idx;
    v.vattr = s->d_vattr;
    v.flags = s->d_flags;
    v.ntris = s->ntris;
    v.nnodes = s->built ? s->nnodes : 0;
    v.root = 0;
    v.tri_base = 0;
    v.isect = s->ctx->isect;
    v.mat = s->d_mat;
    v.cnorm = s->d_cnorm;
    return v;
}

rt_status set_error(rt_status code, const char *msg) { return fail(code, msg); }

bool fast_pow_ok(const rt_light *lights, int32_t n, const rt_material &m)
{
    if (n > RT_MAX_LIGHTS) return false;
    for (int c = 0; c < 3; ++c)
        if (!(m.ks[c] >= 0.0f && m.ks[c] <= 255.0f)) return false;
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c)
            if (!(lights[i].rgb[c] >= 0.0f && lights[i].rgb[c] <= 255.0f) || !(lights[i].d >= 0.0f)) return false;
    return true;
}
rt_status set_cuda_error(cudaError_t e, const char *what) { return cuda_fail(e, what); }

// Copy n bytes of a caller buffer (host or device) into a device buffer.
rt_status stage_in(rt_context *ctx, DevBuf &buf, const void *src, size_t bytes, const void **dev)
{
    if (is_device_ptr(src)) {
        *dev = src;
        return RT_OK;
    }
    RT_CUDA(buf.reserve(bytes), "staging allocation");
    RT_CUDA(cudaMemcpyAsync(buf.ptr, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "host-to-device copy");
    *dev = buf.ptr;
    return RT_OK;
}

rt_status read_counters(rt_context *ctx, Counters *out)
{
    RT_CUDA(cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream),
            "counter readback");
    RT_CUDA(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    *out = *ctx->h_counters;
    return RT_OK;
}

rt_status status_to_error(uint32_t st)
{
    if (st & kStatusStackOverflow) return fail(RT_ERR_STACK_OVERFLOW, "traversal stack overflow");
    if (st & kStatusStepLimit) return fail(RT_ERR_LIMIT, "traversal step limit reached");
    if (st & kStatusBadIndex) return fail(RT_ERR_INTERNAL, "traversal met an index outside the scene");
    return RT_OK;
}

}  // namespace rtc

// =================================================================== C ABI

extern "C" {

const char *rt_last_error_string(void) { return g_last_error.c_str(); }

int32_t rt_version(void) { return 100; }

rt_status rt_ctx_create(int32_t device, rt_context **out)
{
    if (!out) return fail(RT_ERR_INVALID_ARG, "rt_ctx_create: out is NULL");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(RT_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= ndev) return fail(RT_ERR_INVALID_ARG, "rt_ctx_create: device index out of range");
    DeviceGuard g(device);
    if (!g.ok) return fail(RT_ERR_CUDA, "cudaSetDevice failed");
    rt_context *c = new (std::nothrow) rt_context();
    if (!c) return fail(RT_ERR_OUT_OF_MEMORY, "context allocation");
    c->device = device;
    cudaDeviceProp prop;
    RT_CUDA(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    c->sm_count = prop.multiProcessorCount;
    RT_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking), "stream create");
    c->stream = c->own_stream;
    RT_CUDA(cudaMalloc(&c->d_counters, sizeof(Counters)), "counter allocation");
    RT_CUDA(cudaMallocHost(&c->h_counters, sizeof(Counters)), "pinned counter allocation");
    RT_CUDA(cudaMallocHost(&c->h_scratch, 64 * sizeof(int32_t)), "pinned scratch allocation");
    RT_CUDA(cudaEventCreate(&c->ev0), "event create");
    RT_CUDA(cudaEventCreate(&c->ev1), "event create");
    noalloc_context_opened(device);
    *out = c;
    return RT_OK;
}

rt_status rt_ctx_destroy(rt_context *ctx)
{
    if (!ctx) return RT_OK;
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->stage_a.release();
    ctx->stage_b.release();
    ctx->stage_c.release();
    ctx->redo.release();
    soft_release(ctx);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
    if (ctx->h_scratch) cudaFreeHost(ctx->h_scratch);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    noalloc_context_closed(ctx->device);
    delete ctx;
    return RT_OK;
}

rt_status rt_ctx_set_stream(rt_context *ctx, void *stream)
{
    if (!ctx) return fail(RT_ERR_INVALID_ARG, "rt_ctx_set_stream: NULL context");
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return RT_OK;
}

rt_status rt_ctx_set_option(rt_context *ctx, int32_t option, int64_t value)
{
    if (!ctx) return fail(RT_ERR_INVALID_ARG, "rt_ctx_set_option: NULL context");
    if (option == RT_OPT_COUNT_FETCHES) {
        ctx->count_fetches = value != 0;
        return RT_OK;
    }
    if (option == RT_OPT_INTERSECTOR) {
        if (value != RT_ISECT_REFERENCE && value != RT_ISECT_WATERTIGHT)
            return fail(RT_ERR_INVALID_ARG, "rt_ctx_set_option: unknown intersector");
        ctx->isect = (int)value;
        return RT_OK;
    }
    if (option == RT_OPT_MORTON_BITS) {
        if (value != 0 && (value < 10 || value > 21))
            return fail(RT_ERR_INVALID_ARG, "rt_ctx_set_option: Morton bits per axis must be 0 or 10..21");
        ctx->morton_bits = (int)value;
        return RT_OK;
    }
    if (option == RT_OPT_BUILDER) {
        if (value != RT_BUILDER_LBVH && value != RT_BUILDER_PLOC && value != RT_BUILDER_HPLOC)
            return fail(RT_ERR_INVALID_ARG, "rt_ctx_set_option: unknown builder");
        ctx->builder = (int)value;
        return RT_OK;
    }
    if (option == RT_OPT_RENDER_KERNEL) {
        if (value != RT_KERNEL_WAVE && value != RT_KERNEL_PIXEL)
            return fail(RT_ERR_INVALID_ARG, "rt_ctx_set_option: unknown render kernel");
        ctx->render_kernel = (int)value;
        return RT_OK;
    }
    return fail(RT_ERR_INVALID_ARG, "rt_ctx_set_option: unknown option");
}

rt_status rt_ctx_synchronize(rt_context *ctx)
{
    if (!ctx) return fail(RT_ERR_INVALID_ARG, "rt_ctx_synchronize: NULL context");
    DeviceGuard g(ctx->device);
    RT_CUDA(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    return RT_OK;
}

rt_status rt_scene_create(rt_context *ctx, rt_scene **out)
{
    if (!ctx || !out) return fail(RT_ERR_INVALID_ARG, "rt_scene_create: NULL argument");
    rt_scene *s = new (std::nothrow) rt_scene();
    if (!s) return fail(RT_ERR_OUT_OF_MEMORY, "scene allocation");
    s->ctx = ctx;
    *out = s;
    return RT_OK;
}

static void scene_free_geometry(rt_scene *s)
{
    cudaFree(s->d_verts); s->d_verts = nullptr;
    cudaFree(s->d_idx); s->d_idx = nullptr;
    cudaFree(s->d_vattr); s->d_vattr = nullptr;
    cudaFree(s->d_flags); s->d_flags = nullptr;
    cudaFree(s->d_shade); s->d_shade = nullptr;
    cudaFree(s->d_mat); s->d_mat = nullptr; s->mat_max = -1;
    cudaFree(s->d_cnorm); s->d_cnorm = nullptr;
    cudaFree(s->d_nodes); s->d_nodes = nullptr;
    cudaFree(s->d_tris); s->d_tris = nullptr;
    s->temp.release();
    s->built = false;
    s->nnodes = s->tri_slots = s->depth = 0;
}

rt_status rt_scene_destroy(rt_scene *s)
{
    if (!s) return RT_OK;
    DeviceGuard g(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    scene_free_geometry(s);
    delete s;
    return RT_OK;
}

rt_status rt_scene_upload(rt_scene *s, const float *verts, int32_t nverts, const int32_t *tri_idx, int32_t ntris,
                          const float *vattr, const uint32_t *flags)
{
    if (!s) return fail(RT_ERR_INVALID_ARG, "rt_scene_upload: NULL scene");
    if (nverts < 0 || ntris < 0) return fail(RT_ERR_INVALID_ARG, "rt_scene_upload: negative count");
    if ((nverts > 0 && !verts) || (ntris > 0 && !tri_idx)) return fail(RT_ERR_INVALID_ARG, "rt_scene_upload: NULL data");
    if (ntris > (1 << 28)) return fail(RT_ERR_INVALID_ARG, "rt_scene_upload: more than 2^28 triangles");
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    // validate indices on the host when the index buffer is host memory
    const bool idx_dev = is_device_ptr(tri_idx);
    if (!idx_dev) {
        for (int64_t i = 0; i < 3ll * ntris; ++i)
            if (tri_idx[i] < 0 || tri_idx[i] >= nverts)
                return fail(RT_ERR_INVALID_ARG, "rt_scene_upload: vertex index out of range");
    }
    scene_free_geometry(s);
    s->nverts = nverts;
    s->ntris = ntris;
    const size_t nv = (size_t)(nverts > 0 ? nverts : 1), nt = (size_t)(ntris > 0 ? ntris : 1);
    RT_CUDA(cudaMalloc(&s->d_verts, nv * 3 * sizeof(float)), "vertex allocation");
    RT_CUDA(cudaMalloc(&s->d_idx, nt * sizeof(int3)), "index allocation");
    RT_CUDA(cudaMalloc(&s->d_flags, nt * sizeof(uint32_t)), "flag allocation");
    RT_CUDA(cudaMalloc(&s->d_shade, nt * sizeof(ShadeTri)), "shade allocation");
    if (nverts > 0)
        RT_CUDA(cudaMemcpyAsync(s->d_verts, verts, (size_t)nverts * 3 * sizeof(float), cudaMemcpyDefault, ctx->stream),
                "vertex copy");
    if (ntris > 0)
        RT_CUDA(cudaMemcpyAsync(s->d_idx, tri_idx, (size_t)ntris * sizeof(int3), cudaMemcpyDefault, ctx->stream),
                "index copy");
    if (vattr) {
        RT_CUDA(cudaMalloc(&s->d_vattr, nv * 3 * sizeof(float)), "attribute allocation");
        if (nverts > 0)
            RT_CUDA(cudaMemcpyAsync(s->d_vattr, vattr, (size_t)nverts * 3 * sizeof(float), cudaMemcpyDefault,
                                    ctx->stream), "attribute copy");
    }
    if (flags && ntris > 0)
        RT_CUDA(cudaMemcpyAsync(s->d_flags, flags, (size_t)ntris * sizeof(uint32_t), cudaMemcpyDefault, ctx->stream),
                "flag copy");
    else
        RT_CUDA(cudaMemsetAsync(s->d_flags, 0, nt * sizeof(uint32_t), ctx->stream), "flag clear");
    RT_CUDA(cudaStreamSynchronize(ctx->stream), "upload synchronize");
    return RT_OK;
}

rt_status rt_scene_update_vertices(rt_scene *s, const float *verts, int32_t nverts)
{
    if (!s || !verts) return fail(RT_ERR_INVALID_ARG, "rt_scene_update_vertices: NULL argument");
    if (nverts != s->nverts) return fail(RT_ERR_INVALID_ARG, "rt_scene_update_vertices: vertex count changed");
    DeviceGuard g(s->ctx->device);
    if (nverts > 0)
        RT_CUDA(cudaMemcpyAsync(s->d_verts, verts, (size_t)nverts * 3 * sizeof(float), cudaMemcpyDefault,
                                s->ctx->stream), "vertex copy");
    s->built = false;
    return rt_bvh_build(s, nullptr);
}

static int32_t builder_of(int b)
{
    return b == RT_BUILDER_LBVH ? kBuilderLbvh : b == RT_BUILDER_HPLOC ? kBuilderHploc : kBuilderPloc;
}

rt_status rt_bvh_build(rt_scene *s, float *build_ms)
{
    if (!s) return fail(RT_ERR_INVALID_ARG, "rt_bvh_build: NULL scene");
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    s->built = false;
    s->refit = RefitArrays();
    if (build_ms) *build_ms = 0.f;
    if (s->ntris == 0) {
        s->built = true;
        s->nnodes = s->tri_slots = s->depth = 0;
        return RT_OK;
    }
    const size_t nt = (size_t)s->ntris;
    if (!s->d_nodes) RT_CUDA(cudaMalloc(&s->d_nodes, (nt + 1) * sizeof(WideNode)), "node allocation");
    if (!s->d_tris) RT_CUDA(cudaMalloc(&s->d_tris, nt * sizeof(PackedTri)), "triangle allocation");
    const size_t tb = build_temp_bytes(s->ntris);
    RT_CUDA(s->temp.reserve(tb), "build scratch allocation");
    BuildInputs in;
    in.ntris = s->ntris;
    in.verts = s->d_verts;
    in.idx = s->d_idx;
    in.flags = s->d_flags;
    in.shade = s->d_shade;
    in.nodes = s->d_nodes;
    in.tris = s->d_tris;
    in.max_nodes = s->ntris + 1;
    in.sm_count = ctx->sm_count;
    in.host_scratch = ctx->h_scratch;
    in.builder = builder_of(ctx->builder);
    in.morton_bits = ctx->morton_bits;
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    const BuildResult R = build_wide_bvh(in, s->temp.ptr, s->temp.cap, ctx->stream);
    if (R.status != 0) {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "bvh build");
        if (R.status == RT_ERR_STACK_OVERFLOW) return fail(RT_ERR_STACK_OVERFLOW, "bvh build: tree deeper than the traversal stack");
        return fail(R.status, "bvh build failed");
    }
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    RT_CUDA(cudaEventSynchronize(ctx->ev1), "event synchronize");
    RT_CUDA(cudaGetLastError(), "bvh build kernels");
    if (build_ms) cudaEventElapsedTime(build_ms, ctx->ev0, ctx->ev1);
    if (R.tri_slots != s->ntris) return fail(RT_ERR_INTERNAL, "bvh build: triangle count mismatch");
    s->nnodes = R.nodes;
    s->tri_slots = R.tri_slots;
    s->depth = R.depth;
    s->refit = R.refit;
    s->built = true;
    return RT_OK;
}

rt_status rt_scene_refit_vertices(rt_scene *s, const float *verts, int32_t nverts, float *refit_ms)
{
    if (!s || !verts) return fail(RT_ERR_INVALID_ARG, "rt_scene_refit_vertices: NULL argument");
    if (nverts != s->nverts) return fail(RT_ERR_INVALID_ARG, "rt_scene_refit_vertices: vertex count changed");
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_scene_refit_vertices: hierarchy not built");
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    if (refit_ms) *refit_ms = 0.f;
    if (nverts > 0)
        RT_CUDA(cudaMemcpyAsync(s->d_verts, verts, (size_t)nverts * 3 * sizeof(float), cudaMemcpyDefault, ctx->stream),
                "vertex copy");
    if (!s->refit.valid) {   // one triangle or none: nothing to keep, build again
        s->built = false;
        return rt_bvh_build(s, refit_ms);
    }
    s->built = false;
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    const int32_t st = refit_wide_bvh(s->refit, s->d_verts, s->d_idx, s->d_shade, s->d_nodes, s->d_tris,
                                      ctx->h_scratch, ctx->stream);
    if (st != 0) {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "refit");
        return fail(st, "rt_scene_refit_vertices: refit failed");
    }
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    RT_CUDA(cudaEventSynchronize(ctx->ev1), "event synchronize");
    if (refit_ms) cudaEventElapsedTime(refit_ms, ctx->ev0, ctx->ev1);
    s->built = true;
    return RT_OK;
}

rt_status rt_bvh_info(const rt_scene *s, int32_t *nodes, int32_t *tri_slots, int32_t *depth)
{
    if (!s) return fail(RT_ERR_INVALID_ARG, "rt_bvh_info: NULL scene");
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_bvh_info: hierarchy not built");
    if (nodes) *nodes = s->nnodes;
    if (tri_slots) *tri_slots = s->tri_slots;
    if (depth) *depth = s->depth;
    return RT_OK;
}


rt_status rt_bvh_stats_get(const rt_scene *s, rt_bvh_stats *out)
{
    if (!s || !out) return fail(RT_ERR_INVALID_ARG, "rt_bvh_stats_get: NULL argument");
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_bvh_stats_get: hierarchy not built");
    memset(out, 0, sizeof(*out));
    out->nodes = s->nnodes;
    if (s->nnodes == 0) return RT_OK;
    DeviceGuard g(s->ctx->device);
    std::vector<WideNode> h((size_t)s->nnodes);
    RT_CUDA(cudaMemcpy(h.data(), s->d_nodes, h.size() * sizeof(WideNode), cudaMemcpyDeviceToHost), "node download");
    for (const WideNode &n : h)
        for (int k = 0; k < 8; ++k) {
            const uint32_t m = n.meta[k];
            if (m == 0) ++out->empty_slots;
            else if ((n.imask >> k) & 1u) ++out->internal_slots;
            else {
                ++out->leaf_slots;
                const int c = __builtin_popcount(m >> 5);
                if (c >= 1 && c <= 3) ++out->leaf_tris[c];
            }
        }
    return RT_OK;
}

}  // extern "C"

template <bool ANY>
static rt_status trace_common(rt_scene *s, const rt_ray *rays, int32_t n, void *out, const char *name)
{
    if (!s || (n > 0 && (!rays || !out))) return fail(RT_ERR_INVALID_ARG, std::string(name) + ": NULL argument");
    if (n < 0) return fail(RT_ERR_INVALID_ARG, std::string(name) + ": negative ray count");
    if (!s->built) return fail(RT_ERR_NOT_BUILT, std::string(name) + ": hierarchy not built");
    if (n == 0) return RT_OK;
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    const void *d_rays = nullptr;
    rt_status st = stage_in(ctx, ctx->stage_a, rays, (size_t)n * sizeof(rt_ray), &d_rays);
    if (st != RT_OK) return st;
    const size_t out_bytes = ANY ? (size_t)n : (size_t)n * sizeof(rt_hit);
    const bool out_dev = is_device_ptr(out);
    void *d_out = out;
    if (!out_dev) {
        RT_CUDA(ctx->stage_b.reserve(out_bytes), "staging allocation");
        d_out = ctx->stage_b.ptr;
    }
    RT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    const SceneView sv = scene_view(s);
    if (ANY)
        launch_trace_any(sv, (const rt_ray *)d_rays, n, (uint8_t *)d_out, ctx->d_counters, ctx->sm_count, ctx->stream);
    else
        launch_trace_closest(sv, (const rt_ray *)d_rays, n, (rt_hit *)d_out, ctx->d_counters, ctx->sm_count,
                             ctx->stream);
    RT_CUDA(cudaGetLastError(), "trace launch");
    if (!out_dev)
        RT_CUDA(cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, ctx->stream), "device-to-host copy");
    Counters c;
    st = read_counters(ctx, &c);
    if (st != RT_OK) return st;
    return status_to_error(c.status);
}

extern "C" {

rt_status rt_trace_closest(rt_scene *s, const rt_ray *rays, int32_t n, rt_hit *hits)
{
    return trace_common<false>(s, rays, n, hits, "rt_trace_closest");
}

rt_status rt_trace_any(rt_scene *s, const rt_ray *rays, int32_t n, uint8_t *occluded)
{
    return trace_common<true>(s, rays, n, occluded, "rt_trace_any");
}

// Secondary-ray weights of a material: rf and tran each 0 (none) or in
// (0, 1); a refracting material needs a finite positive ri.  Entry points
// without secondary rays take rf = tran = 0 only.
static rt_status check_weights(const rt_material &m, const std::string &w, bool supported)
{
    if (m.rf == 0.0f && m.tran == 0.0f) return RT_OK;
    if (!supported)
        return fail(RT_ERR_INVALID_ARG, w + ": reflective or transparent materials (rf, tran > 0) are rendered by "
                                            "rt_render and rt_render_materials");
    if (!(m.rf >= 0.0f) || !(m.rf < 1.0f)) return fail(RT_ERR_INVALID_ARG, w + ": reflectivity must be 0 or in (0, 1)");
    if (!(m.tran >= 0.0f) || !(m.tran < 1.0f))
        return fail(RT_ERR_INVALID_ARG, w + ": transparency must be 0 or in (0, 1)");
    if (m.tran > 0.0f && !(m.ri > 0.0f && m.ri < 3.0e38f))
        return fail(RT_ERR_INVALID_ARG, w + ": a transparent material needs a finite positive refractive index");
    return RT_OK;
}

// Worst-case ray tree of a set of materials: a ray of power p spawns a
// mirror ray of power p * rf and a refracted ray of power p * tran, each
// traced while its power exceeds 0.1.  With a = the largest rf and b = the
// largest tran, a ray reached by i reflections and j refractions has power
// at most a^i * b^j (times 1 + 2^-24 per binary32 product, hence the slack
// on the threshold), and at most C(i + j, i) rays share (i, j).  The tree
// must stay within RT_MAX_BOUNCES levels and RT_MAX_TREE_RAYS rays.
static rt_status check_tree(const rt_material *m, int32_t n, const std::string &w)
{
    double a = 0.0, b = 0.0;
    for (int32_t k = 0; k < n; ++k) {
        a = std::max(a, (double)m[k].rf);
        b = std::max(b, (double)m[k].tran);
    }
    const double thr = 0.1 * (1.0 - 1.0e-5);
    double rays = 0.0;
    int depth = 0;
    const int lim = 4 * RT_MAX_BOUNCES;
    for (int i = 0; i <= lim; ++i) {
        double binom = 1.0;   // C(i + j, i), j = 0
        for (int j = 0; i + j <= lim; ++j) {
            const double p = std::pow(a, i) * std::pow(b, j);
            if (!(p > thr) && (i + j) > 0) break;
            rays += binom;
            depth = std::max(depth, i + j);
            binom = binom * (double)(i + j + 1) / (double)(j + 1);
        }
    }
    if (depth > RT_MAX_BOUNCES)
        return fail(RT_ERR_INVALID_ARG, w + ": reflectivity and transparency need more than RT_MAX_BOUNCES levels of "
                                            "secondary rays");
    if (rays > (double)RT_MAX_TREE_RAYS)
        return fail(RT_ERR_INVALID_ARG, w + ": reflectivity and transparency allow more than RT_MAX_TREE_RAYS rays "
                                            "per pixel");
    return RT_OK;
}

static rt_status check_material(const rt_material &m, const char *who, bool supported = true)
{
    const std::string w(who);
    const rt_status st = check_weights(m, w, supported);
    if (st != RT_OK || (m.rf == 0.0f && m.tran == 0.0f)) return st;
    return check_tree(&m, 1, w);
}

static rt_status check_camera(const rt_camera *cam)
{
    if (!cam) return fail(RT_ERR_INVALID_ARG, "NULL camera");
    if (cam->xres <= 0 || cam->yres <= 0 || (int64_t)cam->xres * cam->yres > (int64_t)1 << 28)
        return fail(RT_ERR_INVALID_ARG, "camera resolution out of range");
    return RT_OK;
}

// Output staging shared by the two render calls.
struct RenderOut {
    uint8_t *rgb = nullptr;
    int32_t *ids = nullptr;
    int32_t *aux = nullptr;
    bool rgb_host = false, ids_host = false, aux_host = false;
};

static rt_status prepare_outputs(rt_context *ctx, size_t npix, uint8_t *rgb, int32_t *ids, int32_t *aux, RenderOut &o)
{
    o.rgb_host = !is_device_ptr(rgb);
    o.ids_host = ids && !is_device_ptr(ids);
    o.aux_host = aux && !is_device_ptr(aux);
    if (o.rgb_host) {
        RT_CUDA(ctx->stage_a.reserve(npix * 3), "staging allocation");
        o.rgb = (uint8_t *)ctx->stage_a.ptr;
    } else {
        o.rgb = rgb;
    }
    if (o.ids_host) {
        RT_CUDA(ctx->stage_b.reserve(npix * 4), "staging allocation");
        o.ids = (int32_t *)ctx->stage_b.ptr;
    } else {
        o.ids = ids;
    }
    if (o.aux_host) {
        RT_CUDA(ctx->stage_c.reserve(npix * 4), "staging allocation");
        o.aux = (int32_t *)ctx->stage_c.ptr;
    } else {
        o.aux = aux;
    }
    return RT_OK;
}

static rt_status finish_outputs(rt_context *ctx, size_t npix, uint8_t *rgb, int32_t *ids, int32_t *aux,
                                const RenderOut &o, rt_render_stats *stats)
{
    if (o.rgb_host) RT_CUDA(cudaMemcpyAsync(rgb, o.rgb, npix * 3, cudaMemcpyDeviceToHost, ctx->stream), "rgb copy");
    if (o.ids_host) RT_CUDA(cudaMemcpyAsync(ids, o.ids, npix * 4, cudaMemcpyDeviceToHost, ctx->stream), "id copy");
    if (o.aux_host) RT_CUDA(cudaMemcpyAsync(aux, o.aux, npix * 4, cudaMemcpyDeviceToHost, ctx->stream), "aux copy");
    Counters c;
    rt_status st = read_counters(ctx, &c);
    if (st != RT_OK) return st;
    if (stats) {
        stats->primary_rays = (int64_t)c.primary;
        stats->secondary_rays = (int64_t)c.secondary;
        stats->primary_hits = (int64_t)c.hits;
        stats->status = (int32_t)c.status;
        stats->nodes_fetched = (int64_t)c.nodes;
        stats->tris_tested = (int64_t)c.tris;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        stats->device_ms = ms;
    }
    return status_to_error(c.status);
}

rt_status rt_scene_set_normals(rt_scene *s, const float *corner_normals, int32_t ntris)
{
    if (!s) return fail(RT_ERR_INVALID_ARG, "rt_scene_set_normals: NULL scene");
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (!corner_normals) {
        cudaFree(s->d_cnorm);
        s->d_cnorm = nullptr;
        return RT_OK;
    }
    if (ntris != s->ntris) return fail(RT_ERR_INVALID_ARG, "rt_scene_set_normals: ntris differs from the scene's");
    if (!s->d_cnorm)
        RT_CUDA(cudaMalloc(&s->d_cnorm, (size_t)std::max(ntris, 1) * 9 * sizeof(float)), "normal allocation");
    if (ntris > 0)
        RT_CUDA(cudaMemcpyAsync(s->d_cnorm, corner_normals, (size_t)ntris * 9 * sizeof(float), cudaMemcpyDefault,
                                ctx->stream), "normal copy");
    RT_CUDA(cudaStreamSynchronize(ctx->stream), "normal upload synchronize");
    return RT_OK;
}

rt_status rt_scene_set_materials(rt_scene *s, const int32_t *mat_of_tri, int32_t ntris)
{
    if (!s) return fail(RT_ERR_INVALID_ARG, "rt_scene_set_materials: NULL scene");
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (!mat_of_tri) {
        cudaFree(s->d_mat);
        s->d_mat = nullptr;
        s->mat_max = -1;
        return RT_OK;
    }
    if (ntris != s->ntris) return fail(RT_ERR_INVALID_ARG, "rt_scene_set_materials: ntris differs from the scene's");
    int32_t lo = 0, hi = 0;
    const bool dev = is_device_ptr(mat_of_tri);
    if (!dev) {
        for (int32_t i = 0; i < ntris; ++i) {
            lo = std::min(lo, mat_of_tri[i]);
            hi = std::max(hi, mat_of_tri[i]);
        }
        if (lo < 0 || hi >= RT_MAX_MATERIALS)
            return fail(RT_ERR_INVALID_ARG, "rt_scene_set_materials: material index outside 0..RT_MAX_MATERIALS-1");
    }
    int32_t *d = s->d_mat;
    if (!d) RT_CUDA(cudaMalloc(&d, (size_t)std::max(ntris, 1) * sizeof(int32_t)), "material index allocation");
    s->d_mat = d;
    s->mat_max = -1;
    if (ntris > 0)
        RT_CUDA(cudaMemcpyAsync(d, mat_of_tri, (size_t)ntris * sizeof(int32_t), cudaMemcpyDefault, ctx->stream),
                "material index copy");
    if (dev) {
        RT_CUDA(ctx->stage_c.reserve(2 * sizeof(int32_t)), "staging allocation");
        int32_t *range = (int32_t *)ctx->stage_c.ptr;
        launch_index_range(d, ntris, range, ctx->stream);
        RT_CUDA(cudaGetLastError(), "index range launch");
        RT_CUDA(cudaMemcpyAsync(ctx->h_scratch, range, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream),
                "index range readback");
        RT_CUDA(cudaStreamSynchronize(ctx->stream), "stream synchronize");
        lo = ctx->h_scratch[0];
        hi = ctx->h_scratch[1];
        if (lo < 0 || hi >= RT_MAX_MATERIALS) {
            cudaFree(s->d_mat);
            s->d_mat = nullptr;
            return fail(RT_ERR_INVALID_ARG, "rt_scene_set_materials: material index outside 0..RT_MAX_MATERIALS-1");
        }
    }
    RT_CUDA(cudaStreamSynchronize(ctx->stream), "material upload synchronize");
    s->mat_max = hi;
    return RT_OK;
}

// A frame whose materials spawn secondary rays (or differ per triangle):
// the ray-tree kernel.
static rt_status render_tree(rt_scene *s, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                             const rt_material *mats, int32_t nmats, bool per_triangle, uint8_t *rgb_out,
                             int32_t *hit_ids, rt_render_stats *stats)
{
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    const size_t npix = (size_t)camera->xres * (size_t)camera->yres;
    RenderOut o;
    rt_status st = prepare_outputs(ctx, npix, rgb_out, hit_ids, nullptr, o);
    if (st != RT_OK) return st;
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = 0;
    for (int i = 0; i < nlights; ++i) ls.l[i] = make_light_view(lights[i]);
    MaterialTable mt;
    mt.n = nmats;
    for (int i = 0; i < nmats; ++i) mt.m[i] = make_material_view(mats[i]);
    SceneView sv = scene_view(s);
    if (!per_triangle) sv.mat = nullptr;
    RT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    launch_render_tree(sv, make_camera_view(*camera), ls, mt, o.rgb, nullptr, o.ids, ctx->d_counters, ctx->sm_count,
                       ctx->stream, ctx->count_fetches);
    RT_CUDA(cudaGetLastError(), "render launch");
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    return finish_outputs(ctx, npix, rgb_out, hit_ids, nullptr, o, stats);
}

// Lights and a material table for the scene's per-triangle indices.
static rt_status check_table(const rt_scene *s, const rt_light *lights, int32_t nlights, const rt_material *materials,
                             int32_t nmaterials, const std::string &w)
{
    if (nlights < 0 || nlights > RT_MAX_LIGHTS || (nlights > 0 && !lights))
        return fail(RT_ERR_INVALID_ARG, w + ": light count out of range");
    if (nmaterials < 1 || nmaterials > RT_MAX_MATERIALS)
        return fail(RT_ERR_INVALID_ARG, w + ": material count must be 1..RT_MAX_MATERIALS");
    for (int32_t i = 0; i < nmaterials; ++i) {
        const rt_status st = check_weights(materials[i], w, true);
        if (st != RT_OK) return st;
    }
    const rt_status st = check_tree(materials, nmaterials, w);
    if (st != RT_OK) return st;
    if (s->mat_max >= nmaterials) return fail(RT_ERR_INVALID_ARG, w + ": the scene's material indices exceed the table");
    if (!s->built) return fail(RT_ERR_NOT_BUILT, w + ": hierarchy not built");
    return RT_OK;
}

// Layout of ctx->tone: the ToneAcc, a 4-byte word for reductions, then the
// scratch of the tone-mapping kernels.
static constexpr size_t kToneWord = (sizeof(ToneAcc) + 255) / 256 * 256;
static constexpr size_t kToneScratch = kToneWord + 256;

// The tone map of a frame: its parameters checked, and for the histogram
// modes the per-degree resampling of camera::histogram_tone_map
// (camera.cc:1846-1855) computed in the reference's binary32 operations.
static rt_status tone_view(const rt_tone_map *tone, const rt_camera &cam, int32_t fw, int32_t fh, const std::string &w,
                           ToneView &tv)
{
    tv = ToneView{};
    if (!tone) return RT_OK;
    const int m = tone->mode;
    if (!(m == RT_TONE_NONE || m == RT_TONE_GLOBAL_CONTRAST || m == RT_TONE_LOCAL_HISTOGRAM ||
          m == RT_TONE_LOCAL_HUMAN_HISTOGRAM || m == RT_TONE_GLOBAL_NON_LINEAR || m == RT_TONE_GLOBAL_EXPOSURE ||
          m == RT_TONE_GLOBAL_AVG_LUMINANCE || m == RT_TONE_GLOBAL_MAX_LUMINANCE || m == RT_TONE_GLOBAL_FERWERDA ||
          m == RT_TONE_GLOBAL_BILATERAL))
        return fail(RT_ERR_INVALID_ARG, w + ": unsupported tone-mapping mode");
    if (m == RT_TONE_GLOBAL_BILATERAL && !bilateral_grid_fits(fw, fh))
        return fail(RT_ERR_INVALID_ARG, w + ": the bilateral grid of this frame would exceed 2^26 cells");
    const float lim = 3.0e38f;
    if (!(std::fabs(tone->key) < lim && std::fabs(tone->xw) < lim && std::fabs(tone->yw) < lim && tone->gamma >= 0.0f &&
          tone->gamma < lim))
        return fail(RT_ERR_INVALID_ARG, w + ": key, white point and gamma must be finite, gamma >= 0");
    tv.enabled = 1;
    tv.mode = m;
    tv.key = tone->key;
    tv.xw = tone->xw;
    tv.yw = tone->yw;
    tv.desaturate = tone->desaturate ? 1 : 0;
    tv.stretch = tone->stretch ? 1 : 0;
    tv.gamma = tone->gamma;
    if (m == RT_TONE_LOCAL_HISTOGRAM || m == RT_TONE_LOCAL_HUMAN_HISTOGRAM) {
        const float pi = 3.1415926535897932384626433f;
        const float x_m = -cam.w, y_m = -cam.h;   // camera.h:60: x_m = -w, y_m = -h
        const float x_angle = (-2.0f * x_m) / cam.t, y_angle = (-2.0f * y_m) / cam.t;
        const float per_rad = 360.0f / (2.0f * pi);
        const float sx = x_angle * per_rad, sy = y_angle * per_rad;
        if (!(sx >= 2.0f && sy >= 2.0f && sx < 4097.0f && sy < 4097.0f))
            return fail(RT_ERR_INVALID_ARG, w + ": histogram tone mapping needs a view of 2 to 4096 degrees "
                                                "(2w/t and 2h/t in the reference's degree measure)");
        tv.hist_sx = (int32_t)sx;
        tv.hist_sy = (int32_t)sy;
        tv.hist_inc_x = (float)fw / (float)tv.hist_sx;
        tv.hist_inc_y = (float)fh / (float)tv.hist_sy;
    }
    return RT_OK;
}

static int64_t tone_blocks(const ToneView &tv) { return (int64_t)tv.hist_sx * tv.hist_sy; }
static size_t tone_extra(const ToneView &tv, const rt_camera &fine)
{
    return tv.enabled && tv.mode == RT_TONE_GLOBAL_BILATERAL ? bilateral_scratch_bytes(fine.xres, fine.yres) : 0;
}

rt_status rt_tone_map_image(rt_context *ctx, const rt_camera *camera, int32_t aa_x, int32_t aa_y, const float *fimg,
                            const rt_tone_map *tone, uint8_t *rgb_out)
{
    if (!ctx || !fimg || !rgb_out) return fail(RT_ERR_INVALID_ARG, "rt_tone_map_image: NULL argument");
    rt_status st = check_camera(camera);
    if (st != RT_OK) return st;
    if (aa_x < 1 || aa_x > 16 || aa_y < 1 || aa_y > 16)
        return fail(RT_ERR_INVALID_ARG, "rt_tone_map_image: anti-aliasing factors must be 1..16");
    rt_camera fine = *camera;
    fine.xres = camera->xres * aa_x;
    fine.yres = camera->yres * aa_y;
    st = check_camera(&fine);
    if (st != RT_OK) return st;
    ToneView tv;
    st = tone_view(tone, *camera, fine.xres, fine.yres, "rt_tone_map_image", tv);
    if (st != RT_OK) return st;
    DeviceGuard g(ctx->device);
    const size_t npix = (size_t)camera->xres * (size_t)camera->yres;
    const size_t nfine = (size_t)fine.xres * (size_t)fine.yres;
    const void *dimg = nullptr;
    st = stage_in(ctx, ctx->stage_b, fimg, nfine * 3 * sizeof(float), &dimg);
    if (st != RT_OK) return st;
    RenderOut o;
    st = prepare_outputs(ctx, npix, rgb_out, nullptr, nullptr, o);
    if (st != RT_OK) return st;
    RT_CUDA(ctx->tone.reserve(kToneScratch + tone_scratch_bytes((int64_t)nfine, tone_blocks(tv)) + tone_extra(tv, fine)), "scratch allocation");
    RT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    launch_tone_map((const float *)dimg, fine.xres, fine.yres, aa_x, aa_y, tv, o.rgb, (ToneAcc *)ctx->tone.ptr,
                    (char *)ctx->tone.ptr + kToneScratch, ctx->sm_count, ctx->stream);
    RT_CUDA(cudaGetLastError(), "tone-map launch");
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    return finish_outputs(ctx, npix, rgb_out, nullptr, nullptr, o, nullptr);
}

rt_status rt_check_log10(rt_context *ctx, int64_t n, uint64_t seed, int64_t *mismatches, int64_t *undecided)
{
    if (!ctx || !mismatches || !undecided || n < 0) return fail(RT_ERR_INVALID_ARG, "rt_check_log10: bad argument");
    DeviceGuard g(ctx->device);
    RT_CUDA(ctx->tone.reserve(kToneScratch + 256), "scratch allocation");
    unsigned long long *d = (unsigned long long *)((char *)ctx->tone.ptr + kToneWord);
    launch_check_log10(n, seed, d, ctx->sm_count, ctx->stream);
    RT_CUDA(cudaGetLastError(), "check launch");
    RT_CUDA(cudaMemcpyAsync(ctx->h_scratch, d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream),
            "readback");
    RT_CUDA(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    unsigned long long h[2];
    std::memcpy(h, ctx->h_scratch, sizeof(h));
    *mismatches = (int64_t)h[0];
    *undecided = (int64_t)h[1];
    return RT_OK;
}

rt_status rt_sum_sequential_f32(rt_context *ctx, const float *values, int64_t n, float *sum_out)
{
    if (!ctx || !sum_out || (n > 0 && !values)) return fail(RT_ERR_INVALID_ARG, "rt_sum_sequential_f32: NULL argument");
    if (n < 0 || n > ((int64_t)1 << 32)) return fail(RT_ERR_INVALID_ARG, "rt_sum_sequential_f32: n out of range");
    *sum_out = 0.0f;
    if (n == 0) return RT_OK;
    DeviceGuard g(ctx->device);
    const void *dv = nullptr;
    rt_status st = stage_in(ctx, ctx->stage_a, values, (size_t)n * sizeof(float), &dv);
    if (st != RT_OK) return st;
    RT_CUDA(ctx->tone.reserve(kToneScratch + tone_scratch_bytes(n)), "scratch allocation");
    ToneAcc *acc = (ToneAcc *)ctx->tone.ptr;
    uint32_t *mx = (uint32_t *)((char *)ctx->tone.ptr + kToneWord);
    launch_abs_max((const float *)dv, n, mx, ctx->sm_count, ctx->stream);
    RT_CUDA(cudaMemcpyAsync(ctx->h_scratch, mx, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream), "readback");
    RT_CUDA(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    uint32_t bits = (uint32_t)ctx->h_scratch[0];
    if (bits >= 0x7f800000u) return fail(RT_ERR_INVALID_ARG, "rt_sum_sequential_f32: values must be finite");
    if (bits == 0) return RT_OK;   // all zeros: +0
    float max_abs;
    std::memcpy(&max_abs, &bits, sizeof(float));
    launch_sequential_sum((const float *)dv, n, max_abs, acc, (char *)ctx->tone.ptr + kToneScratch, ctx->sm_count,
                          ctx->stream);
    RT_CUDA(cudaGetLastError(), "sum launch");
    RT_CUDA(cudaMemcpyAsync(ctx->h_scratch, &acc->sum_f, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
            "readback");
    RT_CUDA(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    std::memcpy(sum_out, ctx->h_scratch, sizeof(float));
    return RT_OK;
}

rt_status rt_render_tone_mapped(rt_scene *s, const rt_camera *camera, int32_t aa_x, int32_t aa_y,
                                const rt_light *lights, int32_t nlights, const rt_material *materials,
                                int32_t nmaterials, const rt_tone_map *tone, uint8_t *rgb_out, rt_render_stats *stats)
{
    if (!s || !materials || !rgb_out) return fail(RT_ERR_INVALID_ARG, "rt_render_tone_mapped: NULL argument");
    rt_status st = check_camera(camera);
    if (st != RT_OK) return st;
    if (aa_x < 1 || aa_x > 16 || aa_y < 1 || aa_y > 16)
        return fail(RT_ERR_INVALID_ARG, "rt_render_tone_mapped: anti-aliasing factors must be 1..16");
    rt_camera fine = *camera;
    fine.xres = camera->xres * aa_x;
    fine.yres = camera->yres * aa_y;
    st = check_camera(&fine);
    if (st != RT_OK) return st;
    st = check_table(s, lights, nlights, materials, nmaterials, "rt_render_tone_mapped");
    if (st != RT_OK) return st;
    ToneView tv;
    st = tone_view(tone, *camera, fine.xres, fine.yres, "rt_render_tone_mapped", tv);
    if (st != RT_OK) return st;
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    const size_t npix = (size_t)camera->xres * (size_t)camera->yres;
    const size_t nfine = (size_t)fine.xres * (size_t)fine.yres;
    RenderOut o;
    st = prepare_outputs(ctx, npix, rgb_out, nullptr, nullptr, o);
    if (st != RT_OK) return st;
    RT_CUDA(ctx->fimg.reserve(nfine * 3 * sizeof(float)), "float frame allocation");
    RT_CUDA(ctx->tone.reserve(kToneScratch + tone_scratch_bytes((int64_t)nfine, tone_blocks(tv)) + tone_extra(tv, fine)),
            "tone accumulator allocation");
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = 0;
    for (int i = 0; i < nlights; ++i) ls.l[i] = make_light_view(lights[i]);
    MaterialTable mt;
    mt.n = nmaterials;
    for (int i = 0; i < nmaterials; ++i) mt.m[i] = make_material_view(materials[i]);
    RT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    bool secondary = false;
    for (int i = 0; i < nmaterials; ++i) secondary = secondary || materials[i].rf > 0.0f || materials[i].tran > 0.0f;
    if (secondary)
        launch_render_tree(scene_view(s), make_camera_view(fine), ls, mt, nullptr, (float *)ctx->fimg.ptr, nullptr,
                           ctx->d_counters, ctx->sm_count, ctx->stream, ctx->count_fetches);
    else
        launch_render_float(scene_view(s), make_camera_view(fine), ls, mt, (float *)ctx->fimg.ptr, ctx->d_counters,
                            ctx->sm_count, ctx->stream, ctx->count_fetches);
    RT_CUDA(cudaGetLastError(), "render launch");
    launch_tone_map((const float *)ctx->fimg.ptr, fine.xres, fine.yres, aa_x, aa_y, tv, o.rgb, (ToneAcc *)ctx->tone.ptr,
                    (char *)ctx->tone.ptr + kToneScratch, ctx->sm_count, ctx->stream);
    RT_CUDA(cudaGetLastError(), "tone-map launch");
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    return finish_outputs(ctx, npix, rgb_out, nullptr, nullptr, o, stats);
}

rt_status rt_render_image(rt_scene *s, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                          const rt_material *materials, int32_t nmaterials, float *rgb_f32, rt_render_stats *stats)
{
    if (!s || !materials || !rgb_f32) return fail(RT_ERR_INVALID_ARG, "rt_render_image: NULL argument");
    rt_status st = check_camera(camera);
    if (st != RT_OK) return st;
    st = check_table(s, lights, nlights, materials, nmaterials, "rt_render_image");
    if (st != RT_OK) return st;
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    const size_t nsamples = (size_t)camera->xres * (size_t)camera->yres;
    const bool host = !is_device_ptr(rgb_f32);
    float *dst = rgb_f32;
    if (host) {
        RT_CUDA(ctx->fimg.reserve(nsamples * 3 * sizeof(float)), "float frame allocation");
        dst = (float *)ctx->fimg.ptr;
    }
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = 0;
    for (int i = 0; i < nlights; ++i) ls.l[i] = make_light_view(lights[i]);
    MaterialTable mt;
    mt.n = nmaterials;
    for (int i = 0; i < nmaterials; ++i) mt.m[i] = make_material_view(materials[i]);
    bool secondary = false;
    for (int i = 0; i < nmaterials; ++i) secondary = secondary || materials[i].rf > 0.0f || materials[i].tran > 0.0f;
    RT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    if (secondary)
        launch_render_tree(scene_view(s), make_camera_view(*camera), ls, mt, nullptr, dst, nullptr, ctx->d_counters,
                           ctx->sm_count, ctx->stream, ctx->count_fetches);
    else
        launch_render_float(scene_view(s), make_camera_view(*camera), ls, mt, dst, ctx->d_counters, ctx->sm_count,
                            ctx->stream, ctx->count_fetches);
    RT_CUDA(cudaGetLastError(), "render launch");
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    if (host)
        RT_CUDA(cudaMemcpyAsync(rgb_f32, dst, nsamples * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
                "image copy");
    RenderOut o;
    o.rgb_host = false;
    return finish_outputs(ctx, nsamples, nullptr, nullptr, nullptr, o, stats);
}

rt_status rt_render_materials(rt_scene *s, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                              const rt_material *materials, int32_t nmaterials, uint8_t *rgb_out, int32_t *hit_ids,
                              rt_render_stats *stats)
{
    if (!s || !materials || !rgb_out) return fail(RT_ERR_INVALID_ARG, "rt_render_materials: NULL argument");
    rt_status st = check_camera(camera);
    if (st != RT_OK) return st;
    st = check_table(s, lights, nlights, materials, nmaterials, "rt_render_materials");
    if (st != RT_OK) return st;
    bool secondary = false;
    for (int32_t i = 0; i < nmaterials; ++i) secondary |= materials[i].rf != 0.0f || materials[i].tran != 0.0f;
    if (secondary) return render_tree(s, camera, lights, nlights, materials, nmaterials, true, rgb_out, hit_ids, stats);
    if (nmaterials == 1 || !s->d_mat) return rt_render(s, camera, lights, nlights, materials, rgb_out, hit_ids, stats);
    // per-triangle materials without secondary rays: the fused kernel with a table
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    const size_t npix = (size_t)camera->xres * (size_t)camera->yres;
    RenderOut o;
    st = prepare_outputs(ctx, npix, rgb_out, hit_ids, nullptr, o);
    if (st != RT_OK) return st;
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = 1;
    for (int32_t i = 0; i < nmaterials; ++i) ls.fast_pow &= fast_pow_ok(lights, nlights, materials[i]) ? 1 : 0;
    for (int i = 0; i < nlights; ++i) ls.l[i] = make_light_view(lights[i]);
    MaterialTable mt;
    mt.n = nmaterials;
    for (int i = 0; i < nmaterials; ++i) mt.m[i] = make_material_view(materials[i]);
    RT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    launch_render_table(scene_view(s), make_camera_view(*camera), ls, mt, o.rgb, o.ids, ctx->d_counters, ctx->sm_count,
                        ctx->stream, ctx->count_fetches);
    RT_CUDA(cudaGetLastError(), "render launch");
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    return finish_outputs(ctx, npix, rgb_out, hit_ids, nullptr, o, stats);
}

rt_status rt_render(rt_scene *s, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                    const rt_material *material, uint8_t *rgb_out, int32_t *hit_ids, rt_render_stats *stats)
{
    if (!s || !material || !rgb_out) return fail(RT_ERR_INVALID_ARG, "rt_render: NULL argument");
    rt_status st = check_camera(camera);
    if (st != RT_OK) return st;
    if (nlights < 0 || nlights > RT_MAX_LIGHTS || (nlights > 0 && !lights))
        return fail(RT_ERR_INVALID_ARG, "rt_render: light count out of range");
    st = check_material(*material, "rt_render");
    if (st != RT_OK) return st;
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_render: hierarchy not built");
    if (material->rf > 0.0f || material->tran > 0.0f)
        return render_tree(s, camera, lights, nlights, material, 1, false, rgb_out, hit_ids, stats);
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    const size_t npix = (size_t)camera->xres * (size_t)camera->yres;
    RenderOut o;
    st = prepare_outputs(ctx, npix, rgb_out, hit_ids, nullptr, o);
    if (st != RT_OK) return st;
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = fast_pow_ok(lights, nlights, *material) ? 1 : 0;
    for (int i = 0; i < nlights; ++i) ls.l[i] = make_light_view(lights[i]);
    RT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    if (ctx->render_kernel == RT_KERNEL_WAVE)
        launch_render_wave(scene_view(s), make_camera_view(*camera), ls, make_material_view(*material), o.rgb, o.ids,
                           ctx->d_counters, ctx->sm_count, ctx->stream, ctx->count_fetches);
    else
        launch_render(scene_view(s), make_camera_view(*camera), ls, make_material_view(*material), o.rgb, o.ids,
                      ctx->d_counters, ctx->sm_count, ctx->stream, ctx->count_fetches);
    RT_CUDA(cudaGetLastError(), "render launch");
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    return finish_outputs(ctx, npix, rgb_out, hit_ids, nullptr, o, stats);
}

rt_status rt_render_aa(rt_scene *s, const rt_camera *camera, int32_t aa_x, int32_t aa_y, const rt_light *lights,
                       int32_t nlights, const rt_material *material, uint8_t *rgb_out, rt_render_stats *stats)
{
    if (!s || !material || !rgb_out) return fail(RT_ERR_INVALID_ARG, "rt_render_aa: NULL argument");
    rt_status st = check_camera(camera);
    if (st != RT_OK) return st;
    if (aa_x < 1 || aa_x > 16 || aa_y < 1 || aa_y > 16)
        return fail(RT_ERR_INVALID_ARG, "rt_render_aa: anti-aliasing factors must be 1..16");
    rt_camera fine = *camera;   // the supersampled grid the rays are traced on
    fine.xres = camera->xres * aa_x;
    fine.yres = camera->yres * aa_y;
    st = check_camera(&fine);
    if (st != RT_OK) return st;
    if (nlights < 0 || nlights > RT_MAX_LIGHTS || (nlights > 0 && !lights))
        return fail(RT_ERR_INVALID_ARG, "rt_render_aa: light count out of range");
    st = check_material(*material, "rt_render_aa", false);
    if (st != RT_OK) return st;
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_render_aa: hierarchy not built");
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    const size_t npix = (size_t)camera->xres * (size_t)camera->yres;
    RenderOut o;
    st = prepare_outputs(ctx, npix, rgb_out, nullptr, nullptr, o);
    if (st != RT_OK) return st;
    LightSet ls;
    ls.n = nlights;
    ls.fast_pow = fast_pow_ok(lights, nlights, *material) ? 1 : 0;
    for (int i = 0; i < nlights; ++i) ls.l[i] = make_light_view(lights[i]);
    RT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    RT_CUDA(ctx->redo.reserve(npix * sizeof(int32_t)), "redo queue allocation");
    launch_render_aa(scene_view(s), make_camera_view(fine), ls, make_material_view(*material), aa_x, aa_y,
                     camera->xres, camera->yres, o.rgb, (int32_t *)ctx->redo.ptr, ctx->d_counters, ctx->sm_count,
                     ctx->stream, ctx->count_fetches);
    RT_CUDA(cudaGetLastError(), "render launch");
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    return finish_outputs(ctx, npix, rgb_out, nullptr, nullptr, o, stats);
}

rt_status rt_render_ao(rt_scene *s, const rt_camera *camera, const rt_material *material, int32_t samples,
                       float ao_dist, uint32_t seed, uint8_t *rgb_out, int32_t *hit_ids, int32_t *ao_count,
                       rt_render_stats *stats)
{
    if (!s || !material || !rgb_out) return fail(RT_ERR_INVALID_ARG, "rt_render_ao: NULL argument");
    rt_status st = check_camera(camera);
    if (st != RT_OK) return st;
    if (samples < 1 || samples > 64) return fail(RT_ERR_INVALID_ARG, "rt_render_ao: samples must be 1..64");
    if (!(ao_dist > 0.0f)) return fail(RT_ERR_INVALID_ARG, "rt_render_ao: ao_dist must be positive");
    st = check_material(*material, "rt_render_ao", false);
    if (st != RT_OK) return st;
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_render_ao: hierarchy not built");
    rt_context *ctx = s->ctx;
    DeviceGuard g(ctx->device);
    const size_t npix = (size_t)camera->xres * (size_t)camera->yres;
    RenderOut o;
    st = prepare_outputs(ctx, npix, rgb_out, hit_ids, ao_count, o);
    if (st != RT_OK) return st;
    RT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(Counters), ctx->stream), "counter clear");
    RT_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    if (ctx->render_kernel == RT_KERNEL_WAVE)
        launch_render_ao_wave(scene_view(s), make_camera_view(*camera), make_material_view(*material), samples, ao_dist,
                              seed, o.rgb, o.ids, o.aux, ctx->d_counters, ctx->sm_count, ctx->stream,
                              ctx->count_fetches);
    else
        launch_render_ao(scene_view(s), make_camera_view(*camera), make_material_view(*material), samples, ao_dist,
                         seed, o.rgb, o.ids, o.aux, ctx->d_counters, ctx->sm_count, ctx->stream, ctx->count_fetches);
    RT_CUDA(cudaGetLastError(), "render launch");
    RT_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    return finish_outputs(ctx, npix, rgb_out, hit_ids, ao_count, o, stats);
}

}  // extern "C"

// The error setter of the host-only translation units (scene ingest).
rt_status rt_set_error_message(rt_status code, const char *msg) { return rtc::set_error(code, msg); }
