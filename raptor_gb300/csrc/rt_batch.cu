// rt_batch.cu -- many scenes, resolutions and ray mixes in one persistent
// launch.  All scenes of a batch are built in one batched LBVH pass (scene
// id in the top key bits, one sort, one collapse whose level-0 tasks are the
// per-scene roots); every frame of the batch is cut into 32-pixel tiles and
// the tiles of all frames form one device work queue that persistent warps
// drain.  The launch sequence (counter reset + kernel) is captured once in a
// CUDA graph and replayed per batch frame.  Launch shape (threads per block,
// tile shape, tiles claimed per queue access) comes from rt_batch_autotune.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "rt_api_internal.cuh"
#include "rt_build.cuh"
#include "rt_wave.cuh"

using namespace rtc;

namespace rtc {

// A batch job is a FrameJob (rt_wave.cuh).
using BatchJob = FrameJob;

namespace {

// STACK: traversal stack capacity in node groups, chosen by the autotuner
// among the capacities that hold the batch's deepest tree.
template <int TW, int STACK>
__global__ void __launch_bounds__(256, RT_RENDER_MIN_BLOCKS / 2) k_render_batched(const BatchJob *__restrict__ jobs, int32_t njobs,
                                                        int32_t total_items, int32_t chunk, Counters *ctr)
{
    uint32_t status = 0;
    for (;;) {
        const int base = warp_claim(&ctr->work, 32 * chunk);
        if (base >= total_items) break;
        for (int c = 0; c < chunk; ++c) {
            const int item0 = base + 32 * c;
            if (item0 >= total_items) break;
            // job owning this tile: last job with items_begin <= item0 (warp-uniform)
            int lo = 0, hi = njobs - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(&jobs[mid].items_begin) <= item0) lo = mid; else hi = mid - 1;
            }
            const BatchJob &J = jobs[lo];
            int x, y;
            tile_pixel<TW>(item0 - J.items_begin + (threadIdx.x & 31), J.tiles_x, x, y);
            const bool live = (x < J.cam.xres) && (y < J.cam.yres);
            PixelOut po;
            po.hit = false;
            po.secondary = 0;
            if (live) {
                if (J.mode == RT_JOB_AO)
                    po = shade_pixel_ao<false, STACK>(J.sc, J.cam, J.mat, J.ao_samples, J.ao_dist, J.ao_seed, x, y,
                                                      status, nullptr);
                else
                    po = shade_pixel_lights<false, false, STACK>(J.sc, J.cam, J.lights, J.nlights, J.mat, x, y,
                                                                 status, nullptr, J.fast_pow != 0);
                const size_t pix = (size_t)x + (size_t)y * (size_t)J.cam.xres;
                store_rgb(J.rgb, pix, po.c);
                if (J.ids) J.ids[pix] = po.id;
            }
            warp_count(&ctr->primary, live);
            warp_count(&ctr->hits, po.hit);
            warp_add(&ctr->secondary, po.secondary);
        }
    }
    if (status) atomicOr(&ctr->status, status);
}

// Lane-replacement form: every lane carries a pixel of any job and refills
// from the shared queue (rt_wave.cuh).
template <int TW>
__global__ void __launch_bounds__(256, RT_WAVE_MIN_BLOCKS / 2) k_render_batched_wave(const BatchJob *__restrict__ jobs, int32_t njobs,
                                                             int32_t total_items, Counters *ctr)
{
    extern __shared__ LaneShade wave_state[];
    wave_loop<TW, false>(nullptr, jobs, njobs, total_items, wave_state[threadIdx.x], ctr);
}

// Traversal stack capacities the pixel kernel is built for (the wave
// kernel keeps kStackSize).
constexpr int kBatchStacks[3] = {16, 24, kStackSize};

template <int TW, int STACK>
int grid_for(int kernel, int threads, int sm_count)
{
    int per_sm = 0;
    cudaError_t e = (kernel == RT_KERNEL_WAVE)
                        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_batched_wave<TW>, threads,
                                                                        threads * sizeof(LaneShade))
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_batched<TW, STACK>, threads,
                                                                        0);
    if (e != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm * sm_count;
}

}  // namespace
}  // namespace rtc

struct rt_batch {
    rt_context *ctx = nullptr;
    // host-side concatenation of the scenes (global vertex indices)
    std::vector<float> h_verts, h_vattr;
    std::vector<int32_t> h_idx, h_seg;
    std::vector<uint32_t> h_flags;
    std::vector<int32_t> tri_off{0}, vert_off{0};
    std::vector<uint8_t> has_attr;
    // device
    float *d_verts = nullptr, *d_vattr = nullptr;
    int3 *d_idx = nullptr;
    uint32_t *d_flags = nullptr;
    int32_t *d_seg = nullptr;
    ShadeTri *d_shade = nullptr;
    WideNode *d_nodes = nullptr;
    PackedTri *d_tris = nullptr;
    DevBuf temp;
    int32_t nnodes = 0, depth = 0;
    bool built = false;
    // jobs
    std::vector<BatchJob> h_jobs;
    BatchJob *d_jobs = nullptr;
    int32_t total_items = 0;
    // launch configuration and its captured graph
    rt_tune_config cfg{128, 1, 8, RT_KERNEL_PIXEL, 0.f, kStackSize};
    cudaGraphExec_t exec = nullptr;
    cudaStream_t graph_stream = nullptr;
};

namespace {

rt_status bfail(rt_status c, const char *m) { return set_error(c, m); }

#define RT_CUDA_B(call, what)                                  \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return set_cuda_error(_e, what); \
    } while (0)

void free_device(rt_batch *b)
{
    cudaFree(b->d_verts); b->d_verts = nullptr;
    cudaFree(b->d_vattr); b->d_vattr = nullptr;
    cudaFree(b->d_idx); b->d_idx = nullptr;
    cudaFree(b->d_flags); b->d_flags = nullptr;
    cudaFree(b->d_seg); b->d_seg = nullptr;
    cudaFree(b->d_shade); b->d_shade = nullptr;
    cudaFree(b->d_nodes); b->d_nodes = nullptr;
    cudaFree(b->d_tris); b->d_tris = nullptr;
    b->temp.release();
    b->built = false;
}

void drop_graph(rt_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
}

int32_t nscenes(const rt_batch *b) { return (int32_t)b->tri_off.size() - 1; }

// Launch one batch frame directly (the body captured into the graph).
void launch_batch(rt_batch *b, cudaStream_t st, int grid)
{
    cudaMemsetAsync(b->ctx->d_counters, 0, sizeof(Counters), st);
    const int threads = b->cfg.block_threads;
    const int chunk = std::max(1, b->cfg.chunk_tiles);
    const int nj = (int)b->h_jobs.size();
    const size_t smem = (size_t)threads * sizeof(LaneShade);
    if (b->cfg.kernel == RT_KERNEL_WAVE) {
        if (b->cfg.tile_w == 16)
            k_render_batched_wave<16><<<grid, threads, smem, st>>>(b->d_jobs, nj, b->total_items, b->ctx->d_counters);
        else
            k_render_batched_wave<8><<<grid, threads, smem, st>>>(b->d_jobs, nj, b->total_items, b->ctx->d_counters);
    } else {
        Counters *ctr = b->ctx->d_counters;
        const int stack = b->cfg.stack_entries;
#define RT_BATCH_PIXEL(TW, S) k_render_batched<TW, S><<<grid, threads, 0, st>>>(b->d_jobs, nj, b->total_items, chunk, ctr)
        if (b->cfg.tile_w == 16) {
            if (stack == kBatchStacks[0]) RT_BATCH_PIXEL(16, kBatchStacks[0]);
            else if (stack == kBatchStacks[1]) RT_BATCH_PIXEL(16, kBatchStacks[1]);
            else RT_BATCH_PIXEL(16, kBatchStacks[2]);
        } else {
            if (stack == kBatchStacks[0]) RT_BATCH_PIXEL(8, kBatchStacks[0]);
            else if (stack == kBatchStacks[1]) RT_BATCH_PIXEL(8, kBatchStacks[1]);
            else RT_BATCH_PIXEL(8, kBatchStacks[2]);
        }
#undef RT_BATCH_PIXEL
    }
}

// Persistent grid of the configured shape: resident blocks per SM x SMs.
int batch_grid(const rt_batch *b)
{
    const rt_tune_config &c = b->cfg;
    const int sms = b->ctx->sm_count;
    if (c.tile_w == 16) {
        if (c.stack_entries == kBatchStacks[0]) return grid_for<16, kBatchStacks[0]>(c.kernel, c.block_threads, sms);
        if (c.stack_entries == kBatchStacks[1]) return grid_for<16, kBatchStacks[1]>(c.kernel, c.block_threads, sms);
        return grid_for<16, kBatchStacks[2]>(c.kernel, c.block_threads, sms);
    }
    if (c.stack_entries == kBatchStacks[0]) return grid_for<8, kBatchStacks[0]>(c.kernel, c.block_threads, sms);
    if (c.stack_entries == kBatchStacks[1]) return grid_for<8, kBatchStacks[1]>(c.kernel, c.block_threads, sms);
    return grid_for<8, kBatchStacks[2]>(c.kernel, c.block_threads, sms);
}

rt_status make_graph(rt_batch *b)
{
    drop_graph(b);
    cudaStream_t st = b->ctx->stream;
    cudaGraph_t g = nullptr;
    const int grid = batch_grid(b);
    RT_CUDA_B(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "graph capture begin");
    launch_batch(b, st, grid);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (e != cudaSuccess) return set_cuda_error(e, "graph capture end");
    e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->exec = nullptr;
        return set_cuda_error(e, "graph instantiate");
    }
    b->graph_stream = st;
    return RT_OK;
}

// Tile counts depend on the tile shape; recompute the work ranges.
rt_status layout_jobs(rt_batch *b)
{
    int32_t items = 0;
    for (auto &j : b->h_jobs) {
        int tx;
        const int tiles = (b->cfg.tile_w == 16) ? tiles_of<16>(j.cam.xres, j.cam.yres, tx)
                                                 : tiles_of<8>(j.cam.xres, j.cam.yres, tx);
        j.tiles_x = tx;
        j.items_begin = items;
        if ((int64_t)items + (int64_t)tiles * 32 > INT32_MAX) return bfail(RT_ERR_INVALID_ARG, "batch too large");
        items += tiles * 32;
        j.items_end = items;
    }
    b->total_items = items;
    cudaFree(b->d_jobs);
    b->d_jobs = nullptr;
    if (!b->h_jobs.empty()) {
        RT_CUDA_B(cudaMalloc(&b->d_jobs, b->h_jobs.size() * sizeof(BatchJob)), "job table allocation");
        RT_CUDA_B(cudaMemcpy(b->d_jobs, b->h_jobs.data(), b->h_jobs.size() * sizeof(BatchJob), cudaMemcpyHostToDevice),
                  "job table upload");
    }
    return make_graph(b);
}

struct Guard {
    int prev = -1;
    explicit Guard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~Guard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" {

rt_status rt_batch_create(rt_context *ctx, rt_batch **out)
{
    if (!ctx || !out) return bfail(RT_ERR_INVALID_ARG, "rt_batch_create: NULL argument");
    rt_batch *b = new (std::nothrow) rt_batch();
    if (!b) return bfail(RT_ERR_OUT_OF_MEMORY, "batch allocation");
    b->ctx = ctx;
    *out = b;
    return RT_OK;
}

rt_status rt_batch_destroy(rt_batch *b)
{
    if (!b) return RT_OK;
    Guard g(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    drop_graph(b);
    free_device(b);
    cudaFree(b->d_jobs);
    delete b;
    return RT_OK;
}

rt_status rt_batch_add_scene(rt_batch *b, const float *verts, int32_t nverts, const int32_t *tri_idx, int32_t ntris,
                             const float *vattr, const uint32_t *flags, int32_t *scene_index)
{
    if (!b || nverts < 0 || ntris < 0 || (nverts && !verts) || (ntris && !tri_idx))
        return bfail(RT_ERR_INVALID_ARG, "rt_batch_add_scene: invalid argument");
    if (nscenes(b) >= kMaxSegments) return bfail(RT_ERR_INVALID_ARG, "rt_batch_add_scene: too many scenes");
    if ((int64_t)b->tri_off.back() + ntris > (1 << 28)) return bfail(RT_ERR_INVALID_ARG, "batch exceeds 2^28 triangles");
    Guard g(b->ctx->device);
    const int32_t s = nscenes(b);
    const int32_t v0 = b->vert_off.back(), t0 = b->tri_off.back();
    std::vector<float> v((size_t)nverts * 3);
    std::vector<int32_t> t((size_t)ntris * 3);
    if (nverts) RT_CUDA_B(cudaMemcpy(v.data(), verts, v.size() * sizeof(float), cudaMemcpyDefault), "vertex copy");
    if (ntris) RT_CUDA_B(cudaMemcpy(t.data(), tri_idx, t.size() * sizeof(int32_t), cudaMemcpyDefault), "index copy");
    for (size_t i = 0; i < t.size(); ++i) {
        if (t[i] < 0 || t[i] >= nverts) return bfail(RT_ERR_INVALID_ARG, "rt_batch_add_scene: vertex index out of range");
        t[i] += v0;
    }
    b->h_verts.insert(b->h_verts.end(), v.begin(), v.end());
    b->h_idx.insert(b->h_idx.end(), t.begin(), t.end());
    std::vector<float> a((size_t)nverts * 3, 0.f);
    if (vattr && nverts) RT_CUDA_B(cudaMemcpy(a.data(), vattr, a.size() * sizeof(float), cudaMemcpyDefault), "attribute copy");
    b->h_vattr.insert(b->h_vattr.end(), a.begin(), a.end());
    std::vector<uint32_t> f((size_t)ntris, 0u);
    if (flags && ntris) RT_CUDA_B(cudaMemcpy(f.data(), flags, f.size() * sizeof(uint32_t), cudaMemcpyDefault), "flag copy");
    b->h_flags.insert(b->h_flags.end(), f.begin(), f.end());
    b->h_seg.insert(b->h_seg.end(), (size_t)ntris, s);
    b->vert_off.push_back(v0 + nverts);
    b->tri_off.push_back(t0 + ntris);
    b->has_attr.push_back(vattr ? 1 : 0);
    b->built = false;
    if (scene_index) *scene_index = s;
    return RT_OK;
}

rt_status rt_bvh_build_batched(rt_batch *b, float *build_ms)
{
    if (!b) return bfail(RT_ERR_INVALID_ARG, "rt_bvh_build_batched: NULL batch");
    const int32_t ns = nscenes(b);
    if (ns < 1) return bfail(RT_ERR_INVALID_ARG, "rt_bvh_build_batched: no scenes");
    rt_context *ctx = b->ctx;
    Guard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    drop_graph(b);
    free_device(b);
    const size_t nv = std::max<size_t>(1, b->h_verts.size() / 3), nt = std::max<size_t>(1, b->h_idx.size() / 3);
    const int32_t ntris = (int32_t)(b->h_idx.size() / 3);
    RT_CUDA_B(cudaMalloc(&b->d_verts, nv * 3 * sizeof(float)), "vertex allocation");
    RT_CUDA_B(cudaMalloc(&b->d_vattr, nv * 3 * sizeof(float)), "attribute allocation");
    RT_CUDA_B(cudaMalloc(&b->d_idx, nt * sizeof(int3)), "index allocation");
    RT_CUDA_B(cudaMalloc(&b->d_flags, nt * sizeof(uint32_t)), "flag allocation");
    RT_CUDA_B(cudaMalloc(&b->d_seg, nt * sizeof(int32_t)), "segment allocation");
    RT_CUDA_B(cudaMalloc(&b->d_shade, nt * sizeof(ShadeTri)), "shade allocation");
    RT_CUDA_B(cudaMalloc(&b->d_nodes, (nt + ns + 1) * sizeof(WideNode)), "node allocation");
    RT_CUDA_B(cudaMalloc(&b->d_tris, nt * sizeof(PackedTri)), "triangle allocation");
    cudaStream_t st = ctx->stream;
    if (!b->h_verts.empty()) {
        RT_CUDA_B(cudaMemcpyAsync(b->d_verts, b->h_verts.data(), b->h_verts.size() * sizeof(float), cudaMemcpyHostToDevice, st), "upload");
        RT_CUDA_B(cudaMemcpyAsync(b->d_vattr, b->h_vattr.data(), b->h_vattr.size() * sizeof(float), cudaMemcpyHostToDevice, st), "upload");
    }
    if (ntris) {
        RT_CUDA_B(cudaMemcpyAsync(b->d_idx, b->h_idx.data(), b->h_idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st), "upload");
        RT_CUDA_B(cudaMemcpyAsync(b->d_flags, b->h_flags.data(), b->h_flags.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st), "upload");
        RT_CUDA_B(cudaMemcpyAsync(b->d_seg, b->h_seg.data(), b->h_seg.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st), "upload");
    }
    RT_CUDA_B(b->temp.reserve(build_temp_bytes(ntris > 0 ? ntris : 1)), "build scratch allocation");
    BuildInputs in;
    in.ntris = ntris;
    in.verts = b->d_verts;
    in.idx = b->d_idx;
    in.flags = b->d_flags;
    in.shade = b->d_shade;
    in.nodes = b->d_nodes;
    in.tris = b->d_tris;
    in.max_nodes = ntris + ns + 1;
    in.sm_count = ctx->sm_count;
    in.host_scratch = ctx->h_scratch;
    in.builder = ctx->builder == RT_BUILDER_LBVH ? kBuilderLbvh : ctx->builder == RT_BUILDER_HPLOC ? kBuilderHploc : kBuilderPloc;
    in.morton_bits = ctx->morton_bits;
    in.nseg = ns;
    in.seg_of_tri = b->d_seg;
    in.seg_first = b->tri_off.data();
    RT_CUDA_B(cudaEventRecord(ctx->ev0, st), "event record");
    const BuildResult R = build_wide_bvh(in, b->temp.ptr, b->temp.cap, st);
    if (R.status != 0) {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return set_cuda_error(e, "batched bvh build");
        return bfail(R.status, "batched bvh build failed");
    }
    RT_CUDA_B(cudaEventRecord(ctx->ev1, st), "event record");
    RT_CUDA_B(cudaEventSynchronize(ctx->ev1), "event synchronize");
    if (build_ms) cudaEventElapsedTime(build_ms, ctx->ev0, ctx->ev1);
    if (R.tri_slots != ntris) return bfail(RT_ERR_INTERNAL, "batched bvh build: triangle count mismatch");
    b->nnodes = R.nodes;
    b->depth = R.depth;
    b->built = true;
    // refresh scene views of already-set jobs
    for (auto &j : b->h_jobs) {
        const int s = j.sc.root;
        j.sc.nodes = b->d_nodes; j.sc.tris = b->d_tris; j.sc.shade = b->d_shade; j.sc.idx = b->d_idx;
        j.sc.vattr = b->has_attr[s] ? b->d_vattr : nullptr; j.sc.flags = b->d_flags;
        j.sc.ntris = ntris; j.sc.nnodes = b->nnodes; j.sc.tri_base = b->tri_off[s]; j.sc.isect = b->ctx->isect;
    }
    if (!b->h_jobs.empty()) return layout_jobs(b);
    return RT_OK;
}

rt_status rt_batch_set_jobs(rt_batch *b, const rt_job *jobs, int32_t njobs)
{
    if (!b || njobs < 0 || (njobs && !jobs)) return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_jobs: invalid argument");
    if (!b->built) return bfail(RT_ERR_NOT_BUILT, "rt_batch_set_jobs: batch not built");
    Guard g(b->ctx->device);
    std::vector<BatchJob> v;
    v.reserve((size_t)njobs);
    for (int32_t i = 0; i < njobs; ++i) {
        const rt_job &J = jobs[i];
        if (J.scene < 0 || J.scene >= nscenes(b)) return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_jobs: bad scene index");
        if (J.camera.xres <= 0 || J.camera.yres <= 0 || (int64_t)J.camera.xres * J.camera.yres > (1 << 26))
            return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_jobs: resolution out of range");
        if (J.mode != RT_JOB_SHADOW && J.mode != RT_JOB_AO) return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_jobs: bad mode");
        if (J.material.rf != 0.0f || J.material.tran != 0.0f)
            return bfail(RT_ERR_INVALID_ARG,
                         "rt_batch_set_jobs: reflective or transparent materials (rf, tran > 0) are rendered by rt_render");
        if (J.mode == RT_JOB_SHADOW && (J.nlights < 0 || J.nlights > RT_MAX_JOB_LIGHTS))
            return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_jobs: light count out of range");
        if (J.mode == RT_JOB_AO && (J.ao_samples < 1 || J.ao_samples > 64 || !(J.ao_dist > 0.f)))
            return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_jobs: bad AO parameters");
        if (!J.rgb_out || !is_device_ptr(J.rgb_out) || (J.hit_ids && !is_device_ptr(J.hit_ids)))
            return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_jobs: outputs must be device memory");
        BatchJob B;
        memset(&B, 0, sizeof(B));
        const int s = J.scene;
        B.sc.nodes = b->d_nodes; B.sc.tris = b->d_tris; B.sc.shade = b->d_shade; B.sc.idx = b->d_idx;
        B.sc.vattr = b->has_attr[s] ? b->d_vattr : nullptr;
        B.sc.flags = b->d_flags;
        B.sc.ntris = (int32_t)(b->h_idx.size() / 3);
        B.sc.nnodes = b->nnodes;
        B.sc.root = s;
        B.sc.tri_base = b->tri_off[s];
        B.sc.isect = b->ctx->isect;
        B.cam = make_camera_view(J.camera);
        B.mat = make_material_view(J.material);
        B.nlights = J.mode == RT_JOB_SHADOW ? J.nlights : 0;
        for (int l = 0; l < B.nlights; ++l) B.lights[l] = make_light_view(J.lights[l]);
        B.fast_pow = fast_pow_ok(J.lights, B.nlights, J.material) ? 1 : 0;
        B.mode = J.mode;
        B.ao_samples = J.ao_samples;
        B.ao_dist = J.ao_dist;
        B.ao_seed = J.ao_seed;
        B.rgb = J.rgb_out;
        B.ids = J.hit_ids;
        v.push_back(B);
    }
    b->h_jobs.swap(v);
    return layout_jobs(b);
}

rt_status rt_render_batched(rt_batch *b, rt_render_stats *stats)
{
    if (!b) return bfail(RT_ERR_INVALID_ARG, "rt_render_batched: NULL batch");
    if (!b->built) return bfail(RT_ERR_NOT_BUILT, "rt_render_batched: batch not built");
    if (b->h_jobs.empty()) return RT_OK;
    rt_context *ctx = b->ctx;
    Guard g(ctx->device);
    if (!b->exec || b->graph_stream != ctx->stream) {
        rt_status s = make_graph(b);
        if (s != RT_OK) return s;
    }
    RT_CUDA_B(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
    RT_CUDA_B(cudaGraphLaunch(b->exec, ctx->stream), "graph launch");
    RT_CUDA_B(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
    if (!stats) return RT_OK;
    RT_CUDA_B(cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream),
              "counter readback");
    RT_CUDA_B(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    const Counters c = *ctx->h_counters;
    stats->primary_rays = (int64_t)c.primary;
    stats->secondary_rays = (int64_t)c.secondary;
    stats->primary_hits = (int64_t)c.hits;
    stats->status = (int32_t)c.status;
    stats->nodes_fetched = 0;
    stats->tris_tested = 0;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    stats->device_ms = ms;
    return status_to_error(c.status);
}

rt_status rt_batch_set_config(rt_batch *b, const rt_tune_config *cfg)
{
    if (!b || !cfg) return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_config: NULL argument");
    if ((cfg->block_threads != 64 && cfg->block_threads != 128 && cfg->block_threads != 256) ||
        (cfg->tile_w != 8 && cfg->tile_w != 16) || cfg->chunk_tiles < 1 || cfg->chunk_tiles > 16 ||
        (cfg->kernel != RT_KERNEL_WAVE && cfg->kernel != RT_KERNEL_PIXEL))
        return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_config: unsupported configuration");
    if (std::find(std::begin(kBatchStacks), std::end(kBatchStacks), cfg->stack_entries) == std::end(kBatchStacks) ||
        (cfg->kernel == RT_KERNEL_WAVE && cfg->stack_entries != kStackSize))
        return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_config: unsupported traversal stack capacity");
    if (b->built && cfg->stack_entries < b->depth)
        return bfail(RT_ERR_INVALID_ARG, "rt_batch_set_config: traversal stack smaller than the deepest tree");
    Guard g(b->ctx->device);
    b->cfg = *cfg;
    if (b->built && !b->h_jobs.empty()) return layout_jobs(b);
    return RT_OK;
}

rt_status rt_batch_get_config(const rt_batch *b, rt_tune_config *cfg)
{
    if (!b || !cfg) return bfail(RT_ERR_INVALID_ARG, "rt_batch_get_config: NULL argument");
    *cfg = b->cfg;
    return RT_OK;
}

// Time every candidate launch shape on the current jobs (graph replays,
// CUDA events) and keep the fastest.
rt_status rt_batch_autotune(rt_batch *b, int32_t reps, rt_tune_config *best_out)
{
    if (!b) return bfail(RT_ERR_INVALID_ARG, "rt_batch_autotune: NULL batch");
    if (!b->built || b->h_jobs.empty()) return bfail(RT_ERR_NOT_BUILT, "rt_batch_autotune: nothing to tune");
    rt_context *ctx = b->ctx;
    Guard g(ctx->device);
    reps = std::max(1, std::min(reps, 50));
    const int threads[3] = {64, 128, 256};
    const int tiles[2] = {8, 16};
    const int chunks[3] = {1, 2, 4};
    const int kernels[2] = {RT_KERNEL_WAVE, RT_KERNEL_PIXEL};
    rt_tune_config best{128, 1, 8, RT_KERNEL_WAVE, 1e30f, kStackSize};
    for (int kn : kernels)
    for (int tw : tiles)
        for (int th : threads)
            for (int ch : chunks)
            for (int sk : kBatchStacks) {
                if (kn == RT_KERNEL_WAVE && (ch != 1 || sk != kStackSize)) continue;   // the wave form refills per lane
                if (sk < b->depth) continue;   // the stack must hold the deepest tree
                rt_tune_config c{th, ch, tw, kn, 0.f, sk};
                rt_status s = rt_batch_set_config(b, &c);
                if (s != RT_OK) return s;
                RT_CUDA_B(cudaGraphLaunch(b->exec, ctx->stream), "graph launch");   // warm-up
                RT_CUDA_B(cudaEventRecord(ctx->ev0, ctx->stream), "event record");
                for (int r = 0; r < reps; ++r) RT_CUDA_B(cudaGraphLaunch(b->exec, ctx->stream), "graph launch");
                RT_CUDA_B(cudaEventRecord(ctx->ev1, ctx->stream), "event record");
                RT_CUDA_B(cudaEventSynchronize(ctx->ev1), "event synchronize");
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
                c.ms = ms / (float)reps;
                if (c.ms < best.ms) best = c;
            }
    rt_status s = rt_batch_set_config(b, &best);
    if (s != RT_OK) return s;
    if (best_out) *best_out = best;
    return RT_OK;
}

}  // extern "C"
