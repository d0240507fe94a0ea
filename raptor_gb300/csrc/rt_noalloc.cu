// rt_noalloc.cu -- closest-hit tracing for callers that cannot allocate
// device memory.
//
// Some callers must not call cudaMalloc: a renderer embedded in a host
// application whose device memory is owned by another allocator (an engine
// or framework arena that reserves the whole GPU up front), a real-time
// loop that forbids allocation after start-up, or a plugin that is handed a
// fixed memory budget.  rt_trace_closest stages host rays and hits through
// context buffers that grow on demand (cudaMalloc); this entry point instead
// stages everything through one fixed array that lives in the library's own
// device image, so after the first call on a device it touches no allocator.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds it (RT_NOALLOC_SCRATCH_BYTES) until the process exits.  Its
// name is only a host-side stand-in for the symbol; the device address is
// looked up once per device with cudaGetSymbolAddress (on the first call that
// runs on that device, which should therefore come before any stream
// capture) and passed to the copies and the kernel as a plain pointer.  The
// cached address is dropped when the last context on the device is
// destroyed, so a device reset between contexts (which may load the module
// at a new address) is followed by a fresh lookup.
//
// Every call shares the array and leaves its contents behind; the counters
// the kernel needs at zero are cleared by each call.  Calls that overlap on
// the GPU (two host threads, or two contexts on one device, at once) race on
// the array: callers serialise them.  Each call synchronises its stream
// before it returns, so calls made one after another never overlap.
#include <mutex>

#include "rt_api_internal.cuh"

namespace rtc {
namespace {

// Scratch layout: the work/status counters, then the staged rays, then the
// staged hits.
constexpr size_t kCountersBytes = 256;
constexpr size_t kRaysOffset = kCountersBytes;
constexpr size_t kHitsOffset = kRaysOffset + (size_t)RT_NOALLOC_MAX_RAYS * sizeof(rt_ray);
constexpr size_t kScratchBytes = kHitsOffset + (size_t)RT_NOALLOC_MAX_RAYS * sizeof(rt_hit);
static_assert(kScratchBytes == RT_NOALLOC_SCRATCH_BYTES, "scratch size in rtcore.h is out of date");
static_assert(sizeof(Counters) <= kCountersBytes, "counters do not fit their slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
unsigned char *g_scratch_ptr[kMaxDevices] = {};
int g_live_contexts[kMaxDevices] = {};

// Device address of the scratch array on `device` (which must be current).
rt_status scratch_on(int device, unsigned char **out)
{
    if (device < 0 || device >= kMaxDevices)
        return set_error(RT_ERR_INVALID_ARG, "rt_trace_closest_noalloc: device ordinal beyond 63");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[device]) {
        unsigned char *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return set_cuda_error(e, "rt_trace_closest_noalloc: scratch address lookup");
        g_scratch_ptr[device] = p;
    }
    *out = g_scratch_ptr[device];
    return RT_OK;
}

rt_status cuda_check(cudaError_t e, const char *what)
{
    return e == cudaSuccess ? RT_OK : set_cuda_error(e, what);
}

}  // namespace

void noalloc_context_opened(int device)
{
    if (device < 0 || device >= kMaxDevices) return;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    ++g_live_contexts[device];
}

void noalloc_context_closed(int device)
{
    if (device < 0 || device >= kMaxDevices) return;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_live_contexts[device] > 0 && --g_live_contexts[device] == 0) g_scratch_ptr[device] = nullptr;
}

}  // namespace rtc

using namespace rtc;

extern "C" rt_status rt_trace_closest_noalloc(rt_scene *s, const rt_ray *rays, int32_t n, rt_hit *hits)
{
    if (!s || (n > 0 && (!rays || !hits))) return set_error(RT_ERR_INVALID_ARG, "rt_trace_closest_noalloc: NULL argument");
    if (n < 0) return set_error(RT_ERR_INVALID_ARG, "rt_trace_closest_noalloc: negative ray count");
    if (n > RT_NOALLOC_MAX_RAYS)
        return set_error(RT_ERR_INVALID_ARG,
                         "rt_trace_closest_noalloc: more rays than RT_NOALLOC_MAX_RAYS (16384) in one call");
    if (!s->built) return set_error(RT_ERR_NOT_BUILT, "rt_trace_closest_noalloc: hierarchy not built");
    if (n == 0) return RT_OK;
    rt_context *ctx = s->ctx;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return set_error(RT_ERR_CUDA, "rt_trace_closest_noalloc: cudaGetDevice");
    if (prev != ctx->device && cudaSetDevice(ctx->device) != cudaSuccess)
        return set_error(RT_ERR_CUDA, "rt_trace_closest_noalloc: cudaSetDevice");
    struct Restore {
        int dev;
        bool on;
        ~Restore() { if (on) cudaSetDevice(dev); }
    } restore{prev, prev != ctx->device};

    unsigned char *scratch = nullptr;
    rt_status st = scratch_on(ctx->device, &scratch);
    if (st != RT_OK) return st;
    Counters *d_ctr = reinterpret_cast<Counters *>(scratch);
    rt_ray *d_rays = reinterpret_cast<rt_ray *>(scratch + kRaysOffset);
    rt_hit *d_hits = reinterpret_cast<rt_hit *>(scratch + kHitsOffset);
    cudaStream_t stream = ctx->stream;

    st = cuda_check(cudaMemsetAsync(d_ctr, 0, sizeof(Counters), stream), "rt_trace_closest_noalloc: counter clear");
    if (st != RT_OK) return st;
    st = cuda_check(cudaMemcpyAsync(d_rays, rays, (size_t)n * sizeof(rt_ray), cudaMemcpyDefault, stream),
                    "rt_trace_closest_noalloc: ray copy");
    if (st != RT_OK) return st;
    launch_trace_closest(scene_view(s), d_rays, n, d_hits, d_ctr, ctx->sm_count, stream);
    st = cuda_check(cudaGetLastError(), "rt_trace_closest_noalloc: trace launch");
    if (st != RT_OK) return st;
    st = cuda_check(cudaMemcpyAsync(hits, d_hits, (size_t)n * sizeof(rt_hit), cudaMemcpyDefault, stream),
                    "rt_trace_closest_noalloc: hit copy");
    if (st != RT_OK) return st;
    Counters c;
    st = cuda_check(cudaMemcpyAsync(&c, d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, stream),
                    "rt_trace_closest_noalloc: status read");
    if (st != RT_OK) return st;
    st = cuda_check(cudaStreamSynchronize(stream), "rt_trace_closest_noalloc: synchronize");
    if (st != RT_OK) return st;
    return status_to_error(c.status);
}
