// rt_kernels.cuh -- launch interface of the traversal and render kernels.
#pragma once

#include "rt_internal.cuh"

namespace rtc {

constexpr int kTraceThreads = 128;   // 4 warps per block
// Minimum resident blocks per SM the render/trace kernels are compiled for
// (caps registers per thread: 1 -> 255, 6 -> 80, 8 -> 64; 8 measured fastest:
// more resident warps hide the latency of the node loads better than the
// registers the cap spills).
#ifndef RT_WAVE_MIN_BLOCKS
#define RT_WAVE_MIN_BLOCKS RT_RENDER_MIN_BLOCKS   // lane-replacement kernels
#endif
#ifndef RT_RENDER_MIN_BLOCKS
#define RT_RENDER_MIN_BLOCKS 8
#endif
constexpr int kBlocksPerSM = 8;      // persistent grid = SMs x 8 blocks

// Per-launch device counters (zeroed before each launch).
struct Counters {
    int work;                        // next work item (persistent-warp queue)
    uint32_t status;                 // OR of kStatus* bits
    unsigned long long primary;      // primary rays traced
    unsigned long long hits;         // primary hits
    unsigned long long secondary;    // shadow / AO rays traced
    unsigned long long nodes;        // wide nodes fetched (counting kernels only)
    unsigned long long tris;         // triangles tested (counting kernels only)
    int redo;                        // pixels queued for an exact second pass
    unsigned long long drawn;        // random numbers drawn (distributed frames)
};

// Tone-mapping parameters (rt_tone_map) and the per-frame accumulators of
// the tone-mapping kernels (rt_tonemap.cu).
struct ToneView {
    int32_t enabled;   // 0: the downsample and clip alone
    int32_t mode;
    float key, xw, yw;
    int32_t desaturate, stretch;
    float gamma;
    // histogram modes: the frame resampled to hist_sx x hist_sy blocks of
    // hist_inc_x x hist_inc_y samples (one per degree of view)
    int32_t hist_sx, hist_sy;
    float hist_inc_x, hist_inc_y;
    // bilateral mode: each sample's mapped luminance (set by launch_tone_map)
    const float *bil;
};
// The luminance map of the histogram modes (camera::histogram_tone_map).
struct ToneHist {
    int32_t kind;   // 0 black image (no change), 1 linear, 2 contrast, 3 histogram
    float sf, bd_min, bd_max, bw_min, bw_max;
    float cdf[101];
};
struct ToneScalars {
    float sf;    // luminance scale
    float aux;   // non-linear: 1 / (maxY * sf)^2; exposure: maxY * sf
    float k, mp, ms;   // Ferwerda: rod weight, cone and rod scales
};
struct ToneAcc {
    float sum_f;               // binary32 sum of log10 luminance over the counted samples, in sample order
    unsigned long long count;  // samples with luminance >= 3.18e-7
    uint32_t max_bits;         // largest such luminance (float bits)
    uint32_t gmin, gmax;       // mapped-luminance range (order keys), stretch only
    int32_t redo;              // output pixels queued for the exact pass
    float Yi;                  // log-average luminance
    ToneScalars s;
    ToneHist h;
};

struct LightSet {
    int32_t n;
    int32_t fast_pow;   // single-precision specular power + exact re-shade near truncation
    LightView l[RT_MAX_LIGHTS];
};

// The fast specular path is exact in RGB8 when every light intensity and the
// specular colour stay in the reference's 0..255 ranges (shading error bound
// of kTruncGuard).
bool fast_pow_ok(const rt_light *lights, int32_t n, const rt_material &m);

void launch_trace_closest(const SceneView &sc, const rt_ray *rays, int32_t n, rt_hit *hits, Counters *ctr, int sm_count,
                          cudaStream_t st);
void launch_trace_any(const SceneView &sc, const rt_ray *rays, int32_t n, uint8_t *occ, Counters *ctr, int sm_count,
                      cudaStream_t st);
void launch_render(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialView &mat,
                   uint8_t *rgb, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st, bool count = false);
// Float frame (3 floats per pixel, exact) of a frame without secondary rays.
void launch_render_float(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialTable &mt,
                         float *fimg, Counters *ctr, int sm_count, cudaStream_t st, bool count = false);
// k_render with per-triangle materials from a table (no secondary rays).
void launch_render_table(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialTable &mt,
                         uint8_t *rgb, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st, bool count = false);
void launch_render_tree(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialTable &mt,
                        uint8_t *rgb, float *fimg, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st,
                        bool count = false);
void launch_index_range(const int32_t *v, int32_t n, int32_t *out, cudaStream_t st);
// fimg: fw x fh float frame (3 floats per sample, the supersampled grid of
// an ow x oh output with aa_x x aa_y samples per pixel) -> rgb (ow x oh).
// The binary32 sum of v[0..n) in index order, as a sequential loop rounds it
// (into acc->sum_f); max_abs: the largest |v[i]| (launch_abs_max), > 0.
void launch_abs_max(const float *v, int64_t n, uint32_t *out, int sm_count, cudaStream_t st);
void launch_check_log10(int64_t n, uint64_t seed, unsigned long long *out, int sm_count, cudaStream_t st);
void launch_sequential_sum(const float *v, int64_t n, float max_abs, ToneAcc *acc, void *scratch, int sm_count,
                           cudaStream_t st);
// scratch: tone_scratch_bytes(fw * fh, blocks) of device memory (blocks:
// hist_sx * hist_sy of a histogram mode, else 0).
size_t tone_scratch_bytes(int64_t n, int64_t blocks = 0);
// The bilateral mode's extra scratch (after tone_scratch_bytes(n, 0)), and
// whether its grid fits (at most 2^26 cells, 4096 per axis).
size_t bilateral_scratch_bytes(int32_t fw, int32_t fh);
bool bilateral_grid_fits(int32_t fw, int32_t fh);
void launch_tone_map(const float *fimg, int32_t fw, int32_t fh, int32_t aa_x, int32_t aa_y, const ToneView &t,
                     uint8_t *rgb, ToneAcc *acc, void *scratch, int sm_count, cudaStream_t st);
void launch_render_aa(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialView &mat,
                      int32_t aa_x, int32_t aa_y, int32_t out_x, int32_t out_y, uint8_t *rgb, int32_t *redo,
                      Counters *ctr, int sm_count, cudaStream_t st, bool count = false);
void launch_render_ao(const SceneView &sc, const CameraView &cam, const MaterialView &mat, int32_t samples,
                      float ao_dist, uint32_t seed, uint8_t *rgb, int32_t *ids, int32_t *ao_count, Counters *ctr,
                      int sm_count, cudaStream_t st, bool count = false);

// Lane-level ray-replacement variants (rt_wave.cu).
void launch_render_wave(const SceneView &sc, const CameraView &cam, const LightSet &lights, const MaterialView &mat,
                        uint8_t *rgb, int32_t *ids, Counters *ctr, int sm_count, cudaStream_t st, bool count = false);
void launch_render_ao_wave(const SceneView &sc, const CameraView &cam, const MaterialView &mat, int32_t samples,
                           float ao_dist, uint32_t seed, uint8_t *rgb, int32_t *ids, int32_t *ao_count, Counters *ctr,
                           int sm_count, cudaStream_t st, bool count = false);

}  // namespace rtc
