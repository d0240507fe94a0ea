// rt_tonemap.cu -- framebuffer epilogue: the reference's global tone
// mapping (camera::tone_map, raytracer/camera.cc:1124-1463, glare and
// temporal adaptation off), the CIE Yxy -> RGB conversion
// (camera::convert_Yxy_to_rgb, camera.cc:2080-2098), gamma correction
// (camera::gamma_correct, camera.cc:1466-1500) and the anti-aliasing
// downsample with clamp-and-truncate to RGB8 (camera::clip_image_to_rgb,
// camera.h:289-319), on the float frame the ray-tree kernel writes.
//
// Kernels, in stream order:
//   k_tone_terms    one pass over the samples: count and maximum of the
//                   luminances above 3.18e-7, their log10 terms (rounded
//                   once from the exact value: float-float, double for the
//                   few too close to a rounding boundary) and the per-chunk
//                   increments of the exact sequential sum
//   k_tone_coarse   the chunk increments summed over groups of chunks
//   k_tone_sum      one warp: the reference's binary32 sum of the terms,
//                   reproduced exactly, then the mode's scale factors
//   k_hist_blocks   (histogram modes) the luminance averaged per degree of view
//   k_hist_main     (histogram modes) histogram, trimming, cumulative map
//   k_tone_range    (contrast stretch only) minimum and maximum of the
//                   mapped luminance
//   k_tone_final    per output pixel: every sample through the whole
//                   per-pixel chain, averaged, clamped, truncated; single-
//                   precision library calls, pixels near a truncation
//                   boundary queued
//   k_tone_fix      the queued pixels with the library calls evaluated in
//                   double and rounded once (the reference's float results)
// Every per-pixel step uses the reference's binary32 operation order.
#include <cmath>

#include "rt_kernels.cuh"
#include "rt_traverse.cuh"

namespace rtc {
namespace {

constexpr int kToneThreads = 256;

// The reference's float library calls, evaluated in double and rounded
// once (EXACT), or by the single-precision CUDA functions (a few ulp), whose
// pixels are redone exactly when they land near a truncation boundary.
__device__ __forceinline__ float log10_f(float v) { return (float)log10((double)v); }
__device__ __forceinline__ float log_f(float v) { return (float)log((double)v); }
__device__ __forceinline__ float exp_f(float v) { return (float)exp((double)v); }
__device__ __forceinline__ float pow_f(float a, float b) { return (float)pow((double)a, (double)b); }
template <bool EXACT> __device__ __forceinline__ float tl_log10(float v) { return EXACT ? log10_f(v) : log10f(v); }

// ---- log10 of a positive float, correctly rounded, in float-float arithmetic
//
// log10(y) = e * log10(2) + (2 / ln 10) * atanh((m - 1) / (m + 1)) with
// y = m * 2^e, m in [sqrt(1/2), sqrt(2)), so |(m - 1) / (m + 1)| < 0.1716 and
// the atanh series f + f^3/3 + f^5/5 + ... reaches 2^-40 by f^13.  The
// quotient, f^3/3 and the two constant products are carried as float pairs
// (exact products by fma), the smaller terms in float; the result's error
// stays below 2^-33 of its value.  When the float-float value lies within
// that error of a rounding boundary the rounding cannot be decided and the
// function returns false; the caller evaluates log10 in double.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF two_sum(float a, float b)
{
    const float s = xadd(a, b);
    const float bb = xsub(s, a);
    const float err = xadd(xsub(a, xsub(s, bb)), xsub(b, bb));
    return {s, err};
}
__device__ __forceinline__ FF two_prod(float a, float b)
{
    const float p = xmul(a, b);
    return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ FF ff_mul(FF a, FF b)
{
    FF p = two_prod(a.hi, b.hi);
    p.lo = xadd(p.lo, xadd(xmul(a.hi, b.lo), xmul(a.lo, b.hi)));
    return two_sum(p.hi, p.lo);
}
__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    FF s = two_sum(a.hi, b.hi);
    s.lo = xadd(s.lo, xadd(a.lo, b.lo));
    return two_sum(s.hi, s.lo);
}

__device__ __forceinline__ bool log10_ff(float y, float &out)
{
    const uint32_t bits = __float_as_uint(y);
    if (bits < 0x00800000u || bits >= 0x7f800000u) return false;   // zero, subnormal, negative, inf, nan
    int e = (int)(bits >> 23) - 127;
    uint32_t mb = (bits & 0x7fffffu) | 0x3f800000u;
    if (mb > 0x3fb504f3u) {   // m > sqrt(2): halve it
        mb -= 0x00800000u;
        ++e;
    }
    const float m = __uint_as_float(mb);
    const float num = xsub(m, 1.0f);               // exact (Sterbenz)
    const FF den = two_sum(m, 1.0f);
    // f = num / den as a float pair
    const float q = __fdiv_rn(num, den.hi);
    const float rem = xsub(fmaf(-q, den.hi, num), xmul(q, den.lo));
    const FF f = two_sum(q, __fdiv_rn(rem, den.hi));
    // f^3 / 3 as a pair, the rest of the series in float
    const FF f2 = ff_mul(f, f);
    const FF f3 = ff_mul(f2, f);
    const FF third = {__uint_as_float(0x3eaaaaabu), __uint_as_float(0xb22aaaabu)};   // 1/3
    const FF t3 = ff_mul(f3, third);
    const float s = f2.hi;
    const float rest = xmul(xmul(f3.hi, s),
                            xadd(1.0f / 5.0f, xmul(s, xadd(1.0f / 7.0f, xmul(s, xadd(1.0f / 9.0f,
                                 xmul(s, xadd(1.0f / 11.0f, xmul(s, 1.0f / 13.0f)))))))));
    FF at = ff_add(f, t3);
    at = ff_add(at, FF{rest, 0.0f});
    // log10 = 2 * atanh * (1 / ln 10) + e * log10(2)
    const FF inv_ln10 = {__uint_as_float(0x3ede5bd9u), __uint_as_float(0xb22d91afu)};
    const FF log10_2 = {__uint_as_float(0x3e9a209bu), __uint_as_float(0xb2760860u)};
    const FF lm = ff_mul(FF{xmul(2.0f, at.hi), xmul(2.0f, at.lo)}, inv_ln10);
    const FF le = ff_mul(FF{(float)e, 0.0f}, log10_2);
    const FF r = ff_add(le, lm);
    const float rn = xadd(r.hi, r.lo);
    if (rn == 0.0f) {   // y == 1
        out = 0.0f;
        return r.hi == 0.0f && r.lo == 0.0f;
    }
    // distance from the rounding boundaries around rn, against the error bound
    const float d = xadd(xsub(r.hi, rn), r.lo);
    const uint32_t rb = __float_as_uint(rn) & 0x7fffffffu;
    const float ulp = __uint_as_float(((rb >> 23) - 23u) << 23);         // ulp of |rn| (normal rn)
    const bool pow2 = (rb & 0x7fffffu) == 0u;                             // the ulp below |rn| is half of it
    const float up = 0.5f * ulp, down = pow2 ? 0.25f * ulp : 0.5f * ulp;
    const float towards_zero = (rn > 0.0f) ? -d : d;                     // d measured towards 0
    const float margin = xmul(fabsf(rn), 1.1641532e-10f);                 // 2^-33 of the value
    const bool ok = (rb >> 23) > 24u &&
                    ((towards_zero >= 0.0f) ? (towards_zero < down - margin) : (-towards_zero < up - margin));
    out = rn;
    return ok;
}

// log10 rounded once from the exact value: float-float, double where the
// float-float value is too close to a rounding boundary.
__device__ __forceinline__ float log10_cr(float y)
{
    float r;
    if (log10_ff(y, r)) return r;
    return log10_f(y);
}
template <bool EXACT> __device__ __forceinline__ float tl_exp(float v) { return EXACT ? exp_f(v) : expf(v); }
template <bool EXACT> __device__ __forceinline__ float tl_pow(float a, float b) { return EXACT ? pow_f(a, b) : powf(a, b); }

// RGB (0..1) -> CIE luminance scaled by 683 (camera.cc:1149-1151).
__device__ __forceinline__ float lum683(float r, float g, float b)
{
    return xmul(683.0f, xadd(xadd(xmul(0.2126f, r), xmul(0.7151f, g)), xmul(0.0721f, b)));
}

struct Yxy {
    float x, Y, y;
};

// First loop of camera::tone_map for one sample (camera.cc:1137-1193):
// XYZ, the luminance floor, chromaticity, optional desaturation.
template <bool EXACT>
__device__ __forceinline__ Yxy to_yxy(float3 c, const ToneView &t)
{
    const float r = xdiv(c.x, 255.0f), g = xdiv(c.y, 255.0f), b = xdiv(c.z, 255.0f);
    const float X = xmul(683.0f, xadd(xadd(xmul(0.4124f, r), xmul(0.3576f, g)), xmul(0.1805f, b)));
    float Y = lum683(r, g, b);
    const float Z = xmul(683.0f, xadd(xadd(xmul(0.0193f, r), xmul(0.1192f, g)), xmul(0.9505f, b)));
    if (Y < 3.18e-7f) Y = 3.18e-7f;
    const float W = xadd(xadd(Y, X), Z);
    Yxy o;
    o.x = xdiv(X, W);
    o.y = xdiv(Y, W);
    o.Y = Y;
    if (t.desaturate) {
        float s;
        const float l = tl_log10<EXACT>(Y);
        if (l < -2.0f) {
            s = 0.0f;
        } else if (l < 0.6f) {
            const float q = xdiv(xadd(l, 2.0f), 2.6f);
            const float q2 = xmul(q, q);
            s = xsub(xmul(3.0f, q2), xmul(xmul(2.0f, q), q2));
        } else {
            s = 1.0f;
        }
        const float V = xmul(1700.0f, xadd(xadd(xmul(0.01477f, r), xmul(0.497f, g)), xmul(0.631f, b)));
        const float third = 1.0f / 3.0f;
        const float one_s = xsub(1.0f, s);
        o.x = xadd(xmul(one_s, t.xw), xmul(s, xsub(xadd(o.x, t.xw), third)));
        o.y = xadd(xmul(one_s, t.yw), xmul(s, xsub(xadd(o.y, t.yw), third)));
        o.Y = xadd(xmul(xmul(0.4468f, one_s), V), xmul(s, Y));
    }
    return o;
}

// The mode's luminance scaling (camera.cc:1276-1425) of one sample.
template <bool EXACT> __device__ __forceinline__ float tl_log(float v) { return EXACT ? log_f(v) : logf(v); }

// camera::histogram_tone_map's final loop (camera.cc:2040-2056) for one
// luminance, and its linear and contrast fallbacks.
template <bool EXACT>
__device__ __forceinline__ float map_hist(float g, const ToneHist &h)
{
    switch (h.kind) {
    case 1:
        return xadd(xmul(g, h.sf), h.bd_min);
    case 2:
        return xmul(g, h.sf);
    case 3: {
        if (!(g > 0.0f)) return g;
        const float bw = tl_log<EXACT>(g);
        float bf = xmul(xdiv(xsub(bw, h.bw_min), xsub(h.bw_max, h.bw_min)), 100.0f);
        bf = (bf < 0.0f) ? 0.0f : bf;            // std::max(bf, 0), then std::min(., bins)
        bf = (100.0f < bf) ? 100.0f : bf;
        const int b0 = (int)bf;
        const int b1 = (b0 + 1 < 100) ? b0 + 1 : 100;
        const float s = xsub(bf, (float)b0);
        const float pbw = xadd(xmul(xsub(1.0f, s), h.cdf[b0]), xmul(s, h.cdf[b1]));
        const float bde = xadd(h.bd_min, xmul(xsub(h.bd_max, h.bd_min), pbw));
        return xdiv(tl_exp<EXACT>(bde), 300.0f);
    }
    default:
        return g;
    }
}

template <bool EXACT>
__device__ __forceinline__ float map_lum(float g, const ToneView &t, const ToneScalars &k, const ToneHist &hh)
{
    switch (t.mode) {
    case RT_TONE_LOCAL_HISTOGRAM:
    case RT_TONE_LOCAL_HUMAN_HISTOGRAM:
        return map_hist<EXACT>(g, hh);
    case RT_TONE_GLOBAL_NON_LINEAR:
        g = xmul(g, k.sf);
        if (k.aux != 0.0f) g = xmul(g, xdiv(xadd(1.0f, xmul(g, k.aux)), xadd(1.0f, g)));
        return g;
    case RT_TONE_GLOBAL_EXPOSURE:
        g = xmul(g, k.sf);
        if (k.aux != 0.0f) g = xsub(1.0f, tl_exp<EXACT>(-g));
        return g;
    case RT_TONE_GLOBAL_FERWERDA: {
        const float ldp = xmul(k.mp, g), lds = xmul(k.ms, g);
        return xmul(1.0f / 800.0f, xadd(ldp, xmul(k.k, lds)));
    }
    default:   // none, contrast, average and maximum luminance: one scale
        return xmul(g, k.sf);
    }
}

// Yxy -> RGB in 0..255 (camera.cc:2085-2096), then gamma (camera.cc:1470-1497).
// powed (nullable) is set when a gamma power is evaluated on a value
// strictly between the clamp bounds (a clamped 0 or 1 gives the same
// channel in single and double precision).
template <bool EXACT>
__device__ __forceinline__ float3 to_rgb(float x, float Y, float y, float gamma, bool *powed = nullptr)
{
    const float X = xdiv(xmul(x, Y), y);
    const float Z = xdiv(xmul(xsub(xsub(1.0f, x), y), Y), y);
    float3 c;
    c.x = xadd(xadd(xmul(826.353f, X), xmul(-391.986f, Y)), xmul(-127.143f, Z));
    c.y = xadd(xadd(xmul(-247.0695f, X), xmul(478.329f, Y)), xmul(10.5825f, Z));
    c.z = xadd(xadd(xmul(14.2035f, X), xmul(-52.02f, Y)), xmul(269.535f, Z));
    if (gamma > 0.0f) {
        float v[3] = {xdiv(c.x, 255.0f), xdiv(c.y, 255.0f), xdiv(c.z, 255.0f)};
        const bool plain = fabsf(xsub(gamma, 2.2f)) > 0.001f;
        const bool srgb = !plain && fabsf(xsub(gamma, 1.0f)) > 0.001f;
        const float inv = xdiv(1.0f, gamma);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float a = v[i];
            a = (a < 0.0f) ? 0.0f : a;   // std::max(a, 0), then std::min(., 1)
            a = (1.0f < a) ? 1.0f : a;
            if (powed && ((plain && a > 0.0f && a < 1.0f) || (srgb && a > 0.0031308f && a < 1.0f))) *powed = true;
            if (plain) a = tl_pow<EXACT>(a, inv);
            else if (srgb)
                a = (a <= 0.0031308f) ? xmul(12.92f, a) : xsub(xmul(1.055f, tl_pow<EXACT>(a, 1.0f / 2.4f)), 0.055f);
            v[i] = a;
        }
        c = make_float3(xmul(v[0], 255.0f), xmul(v[1], 255.0f), xmul(v[2], 255.0f));
    }
    return c;
}

// ---- camera::histogram_tone_map (camera.cc:1843-2062)

// The block bounds of camera.cc:1856-1880 as the reference's running sums
// produce them (x1 = min(w - 1, x1 + inc), x0 = the previous x1): thread 0
// the columns, thread 1 the rows, into bx (2 * hist_sx floats) and by.
__global__ void k_hist_bounds(int32_t fw, int32_t fh, ToneView t, float *__restrict__ bx, float *__restrict__ by)
{
    const bool cols = threadIdx.x == 0;
    if (threadIdx.x > 1) return;
    const int n = cols ? t.hist_sx : t.hist_sy;
    const float inc = cols ? t.hist_inc_x : t.hist_inc_y;
    const float vmax = xsub((float)(cols ? fw : fh), 1.0f);
    float *out = cols ? bx : by;
    float v0 = 0.0f, v1 = inc;
    for (int q = 0; q < n; ++q) {
        out[2 * q] = v0;
        out[2 * q + 1] = v1;
        v0 = v1;
        const float nv = xadd(v1, inc);
        v1 = (nv < vmax) ? nv : vmax;   // std::min(res - 1, v1 + inc)
    }
}

// The frame's luminance averaged over one block per degree of view
// (camera.cc:1856-1880): block (i, j) sums the samples of rows
// int(y0)..int(y1) and columns int(x0)..int(x1) in that order.  One thread
// per block.
__global__ void __launch_bounds__(kToneThreads) k_hist_blocks(const float *__restrict__ fimg, int32_t fw, int32_t fh,
                                                              ToneView t, const float *__restrict__ bx,
                                                              const float *__restrict__ by, float *__restrict__ blocks)
{
    const int64_t nb = (int64_t)t.hist_sx * t.hist_sy;
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(b % t.hist_sx), j = (int)(b / t.hist_sx);
        const float x0 = bx[2 * i], x1 = bx[2 * i + 1], y0 = by[2 * j], y1 = by[2 * j + 1];
        float acc = 0.0f;
        for (int y = (int)y0; y <= (int)y1; ++y)
            for (int x = (int)x0; x <= (int)x1; ++x) {
                const int64_t s = (int64_t)y * fw + x;
                acc = xadd(acc, to_yxy<true>(make_float3(fimg[3 * s], fimg[3 * s + 1], fimg[3 * s + 2]), t).Y);
            }
        blocks[b] = xdiv(acc, xmul(xadd(xsub(x1, x0), 1.0f), xadd(xsub(y1, y0), 1.0f)));
    }
}

// camera::just_noticable_difference (camera.cc:1814-1840).
__device__ __forceinline__ float jnd(float La)
{
    const float l = log10_f(La);
    float t;
    if (l < -3.94f) t = -2.86f;
    else if (l < -1.44f) t = xsub(pow_f(xadd(xmul(0.405f, l), 1.6f), 2.18f), 2.86f);
    else if (l < -0.0184f) t = xsub(l, 0.395f);
    else if (l < 1.9f) t = xsub(pow_f(xadd(xmul(0.249f, l), 0.65f), 2.7f), 0.72f);
    else t = xsub(l, 1.255f);
    return pow_f(10.0f, t);
}

// The rest of histogram_tone_map up to the final per-pixel loop, in one
// block of 128 threads: range of the positive blocks, the linear and
// contrast fallbacks, a 100-bin histogram of log luminance, and the
// trimming iterations (each bin's ceiling in its own thread; counts and the
// cumulative histogram are integers below 2^24, so their binary32 running
// sums are exact in any order).  Iterations are capped at 10,000; the
// reference's loop ends far sooner (each pass trims a bin down to its
// ceiling).
__global__ void __launch_bounds__(128) k_hist_main(const float *__restrict__ blocks, ToneView t, ToneAcc *acc)
{
    __shared__ int his[101];
    __shared__ float cdf[101];
    __shared__ int s_cnt, s_trim;
    __shared__ uint32_t s_min, s_max;
    const int tid = threadIdx.x;
    const int64_t nb = (int64_t)t.hist_sx * t.hist_sy;
    if (tid == 0) {
        s_cnt = 0;
        s_min = 0x7f7fffffu;   // FLT_MAX
        s_max = 0u;
    }
    if (tid <= 100) {
        his[tid] = 0;
        cdf[tid] = 0.0f;
    }
    __syncthreads();
    int cnt = 0;
    uint32_t mn = 0x7f7fffffu, mx = 0u;
    for (int64_t b = tid; b < nb; b += blockDim.x) {
        const float v = blocks[b];
        if (v > 0.0f) {
            mn = min(mn, __float_as_uint(v));   // positive: bit order is value order
            mx = max(mx, __float_as_uint(v));
            ++cnt;
        }
    }
    atomicAdd(&s_cnt, cnt);
    atomicMin(&s_min, mn);
    atomicMax(&s_max, mx);
    __syncthreads();
    ToneHist &H = acc->h;
    int pix_gt0 = s_cnt;
    float lw_min = __uint_as_float(s_min), lw_max = __uint_as_float(s_max);
    if (!(lw_min > 0.0f)) {   // never: lw_min starts at FLT_MAX and only takes positive values
        if (tid == 0) H.kind = 0;
        return;
    }
    lw_min = (lw_min < 1.0e-4f) ? 1.0e-4f : lw_min;   // std::max(lw_min, min_lum)
    const float bw_min = log_f(lw_min);
    float bw_max = log_f(lw_max);
    if (bw_max == bw_min) bw_max = xadd(bw_max, xmul(0.0001f, fabsf(bw_max)));
    const float ld_max = 300.0f;
    const float bd_max = log_f(ld_max), bd_min = log_f(1.0f);
    if (tid == 0) {
        H.bd_min = bd_min;
        H.bd_max = bd_max;
        H.bw_min = bw_min;
        H.bw_max = bw_max;
    }
    if (xsub(bd_max, bd_min) > xsub(bw_max, bw_min)) {
        if (tid == 0) {
            H.kind = 1;
            H.sf = xdiv(xsub(bd_max, bd_min), xsub(bw_max, bw_min));
        }
        return;
    }
    for (int64_t b = tid; b < nb; b += blockDim.x) {
        const float v = blocks[b];
        if (v > 0.0f) {
            int bin = (int)xmul(xdiv(xsub(log_f(v), bw_min), xsub(bw_max, bw_min)), 100.0f) + 1;
            bin = bin < 0 ? 0 : (bin > 100 ? 100 : bin);
            atomicAdd(&his[bin], 1);
        }
    }
    __syncthreads();
    if (tid == 0) {
        float sum = 0.0f;
        for (int i = 1; i <= 100; ++i) {
            sum = xadd(sum, (float)his[i]);
            cdf[i] = xdiv(sum, (float)pix_gt0);
        }
    }
    __syncthreads();
    const float tolerance = xmul(0.025f, (float)pix_gt0);
    const float bin_step = xdiv(xsub(bw_max, bw_min), 100.0f);
    const float lw_step = xmul(1.0f / 100.0f, xsub(bw_max, bw_min));
    const bool human = t.mode == RT_TONE_LOCAL_HUMAN_HISTOGRAM;
    for (int iter = 0; iter < 10000; ++iter) {
        if ((float)pix_gt0 < tolerance) {
            if (tid == 0) {
                const float num = xadd(1.219f, pow_f(xmul(ld_max, 0.5f), 0.4f));
                const float den = xadd(1.219f, pow_f(acc->Yi, 0.4f));
                H.kind = 2;
                H.sf = xmul(xdiv(1.0f, ld_max), pow_f(xdiv(num, den), 2.5f));
            }
            return;
        }
        if (tid == 0) s_trim = 0;
        __syncthreads();
        const int i = tid + 1;
        if (i <= 100) {
            float ceiling = xdiv(xmul((float)pix_gt0, bin_step), xsub(bd_max, bd_min));
            if (human) {
                const float bde = xadd(bd_min, xmul(xsub(bd_max, bd_min), cdf[i]));
                const float ld = exp_f(bde);
                const float bw = xadd(xmul((float)i, lw_step), bw_min);
                const float lw = exp_f(bw);
                ceiling = xmul(ceiling, xdiv(xmul(jnd(ld), lw), xmul(jnd(lw), ld)));
            }
            if ((float)his[i] > ceiling) {
                atomicAdd(&s_trim, his[i] - (int)ceiling);
                his[i] = (int)ceiling;
            }
        }
        __syncthreads();
        if (tid == 0) {
            int p = 0;
            for (int k = 1; k <= 100; ++k) p += his[k];
            s_cnt = p;
            float sum = 0.0f;
            for (int k = 1; k <= 100; ++k) {
                sum = xadd(sum, (float)his[k]);
                cdf[k] = xdiv(sum, (float)p);
            }
        }
        __syncthreads();
        pix_gt0 = s_cnt;
        const int trimmings = s_trim;
        __syncthreads();
        if (!((float)trimmings > tolerance)) break;
    }
    if (tid <= 100) H.cdf[tid] = cdf[tid];
    if (tid == 0) H.kind = 3;
}

// Order-preserving key of a float for unsigned atomics (no NaNs here).
__device__ __forceinline__ uint32_t order_key(float f)
{
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// ---- the log-average luminance, summed as the reference sums it
//
// The reference adds log10(Y) of every counted sample to a binary32 sum in
// sample order (camera.cc:1158).  That sum is reproduced exactly: while the
// running sum S stays in one binade [2^e, 2^(e+1)), every addition rounds
// to a multiple of u = 2^(e-23), so S + a_i = S + u * rne(a_i / u) as long
// as no rne is a tie and no partial sum leaves the binade.  k_tone_terms
// writes the terms and, per chunk of kSumChunk terms and for each of 32
// candidate binades, the sums of the positive and of the negative rne
// increments and a tie flag; k_tone_sum walks the chunks in order with one
// warp, applying a chunk in one step when its increments provably keep S
// inside S's binade and adding its terms one by one otherwise (the first
// chunk, binade changes, ties).  Uncounted samples contribute +0, which
// leaves S unchanged.
constexpr int kSumChunk = 512;
constexpr int kSumThreads = 128;
constexpr int kSumPerThread = kSumChunk / kSumThreads;

struct ChunkSum {
    int32_t pos, neg;   // sums of the positive / negative increments in units of u, saturated at +-2^30
    int32_t tie, pad;
};

// Increments and their sums beyond +-2^24 units can never be applied (the
// sum would leave the binade), so they are stored saturated.
constexpr int32_t kSat = 1 << 30;
__device__ __forceinline__ int32_t sat32(long long v) { return v > kSat ? kSat : (v < -kSat ? -kSat : (int32_t)v); }

// values non-null: the terms are given (rt_sum_sequential_f32) instead of
// derived from the frame.
__global__ void __launch_bounds__(kSumThreads) k_tone_terms(const float *__restrict__ fimg,
                                                            const float *__restrict__ values, int64_t n, int32_t e_lo,
                                                            float *__restrict__ terms, ChunkSum *__restrict__ rec,
                                                            ToneAcc *acc)
{
    __shared__ long long s_pos[32], s_neg[32];
    __shared__ int32_t s_tie[32];
    if (threadIdx.x < 32) {
        s_pos[threadIdx.x] = 0;
        s_neg[threadIdx.x] = 0;
        s_tie[threadIdx.x] = 0;
    }
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSumChunk;
    float a[kSumPerThread];
    uint32_t cnt = 0, maxb = 0;
#pragma unroll
    for (int t = 0; t < kSumPerThread; ++t) {
        const int64_t i = base + t * kSumThreads + threadIdx.x;
        a[t] = 0.0f;
        if (i < n && values) {
            a[t] = values[i];
        } else if (i < n) {
            const float r = xdiv(fimg[3 * i], 255.0f), g = xdiv(fimg[3 * i + 1], 255.0f),
                        b = xdiv(fimg[3 * i + 2], 255.0f);
            const float Y = lum683(r, g, b);
            if (!(Y < 3.18e-7f)) {
                ++cnt;
                maxb = max(maxb, __float_as_uint(Y));   // Y > 0: bit order is value order
                a[t] = log10_cr(Y);
            }
        }
        terms[i] = a[t];   // the padding of the last chunk holds +0
    }
    // Per binade ei: the warp's sums of the positive and negative rounded
    // increments (one redux each) and its tie flags (bit ei, one redux for
    // all 32); lane ei keeps binade ei's sums.  A lane's own sums (4 terms of
    // |q| <= 2^26) fit in int32; each is clamped to +-2^25 before the warp
    // sum, so that sum stays below 2^30 and is exact unless some lane was
    // clamped, in which case it is >= 2^25 in magnitude: a record that large
    // never applies, whatever its exact value.
    const int lane = threadIdx.x & 31;
    int32_t my_pos = 0, my_neg = 0;
    uint32_t ties = 0;
    for (int ei = 0; ei < 32; ++ei) {
        int32_t pos = 0, neg = 0;
#pragma unroll
        for (int t = 0; t < kSumPerThread; ++t) {
            const float k = ldexpf(a[t], 23 - (e_lo + ei));   // exact: a power-of-two scale
            int32_t q;
            if (fabsf(k) < 33554432.0f) {                      // |k| < 2^25
                q = __float2int_rn(k);                         // round to nearest, ties to even
                if (xsub(k, floorf(k)) == 0.5f) ties |= 1u << ei;
            } else {
                q = (k > 0.0f) ? (1 << 26) : -(1 << 26);       // too large to apply: saturates the sums
            }
            if (q > 0) pos += q;
            else neg += q;
        }
        const int32_t wpos = __reduce_add_sync(0xffffffffu, min(pos, 1 << 25));
        const int32_t wneg = __reduce_add_sync(0xffffffffu, max(neg, -(1 << 25)));
        if (lane == ei) {
            my_pos = wpos;
            my_neg = wneg;
        }
    }
    ties = __reduce_or_sync(0xffffffffu, ties);
    atomicAdd((unsigned long long *)&s_pos[lane], (unsigned long long)(long long)my_pos);
    atomicAdd((unsigned long long *)&s_neg[lane], (unsigned long long)(long long)my_neg);
    if ((ties >> lane) & 1u) atomicOr(&s_tie[lane], 1);
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        maxb = max(maxb, __shfl_xor_sync(0xffffffffu, maxb, o));
    }
    if (lane == 0 && cnt) {
        atomicAdd(&acc->count, (unsigned long long)cnt);
        atomicMax(&acc->max_bits, maxb);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        ChunkSum c;
        c.pos = sat32(s_pos[threadIdx.x]);
        c.neg = sat32(s_neg[threadIdx.x]);
        c.tie = s_tie[threadIdx.x];
        c.pad = 0;
        rec[(int64_t)blockIdx.x * 32 + threadIdx.x] = c;
    }
}

// The scale factors of camera::tone_map's mode branch (camera.cc:1203-1425)
// from the log-luminance sum, the counted samples and the maximum.
__device__ void tone_scalars(const ToneView &t, ToneAcc *acc)
{
    float Yi = 0.0f;
    if (acc->count) Yi = xdiv(acc->sum_f, (float)acc->count);
    Yi = pow_f(10.0f, Yi);
    acc->Yi = Yi;
    float maxY = __uint_as_float(acc->max_bits);
    ToneScalars k;
    k.sf = 1.0f;
    k.aux = 0.0f;
    k.k = k.mp = k.ms = 0.0f;
    switch (t.mode) {
    case RT_TONE_GLOBAL_CONTRAST: {
        const float Yw = 300.0f;
        const float num = xadd(1.219f, pow_f(xmul(Yw, 0.5f), 0.4f));
        const float den = xadd(1.219f, pow_f(Yi, 0.4f));
        k.sf = xmul(xdiv(1.0f, Yw), pow_f(xdiv(num, den), 2.5f));
        break;
    }
    case RT_TONE_GLOBAL_NON_LINEAR:
        k.sf = xdiv(t.key, Yi);
        maxY = xmul(maxY, k.sf);
        k.aux = xdiv(1.0f, xmul(maxY, maxY));
        break;
    case RT_TONE_GLOBAL_EXPOSURE:
        k.sf = xdiv(t.key, Yi);
        k.aux = xmul(maxY, k.sf);
        break;
    case RT_TONE_GLOBAL_AVG_LUMINANCE:
        // the reference accumulates its RGB average only in exposure mode
        // (camera.cc:1142), so here it is zero and the scale stays 1
        k.sf = 1.0f;
        break;
    case RT_TONE_GLOBAL_MAX_LUMINANCE:
        k.sf = xdiv(t.key, maxY);
        break;
    case RT_TONE_GLOBAL_FERWERDA: {
        const float log_lda = log_f(xmul(800.0f, 0.5f));
        const float log_la = log_f(Yi);
        float tp, ts;
        if (log_la <= -2.6f) tp = -0.72f;
        else if (log_la <= 1.9f) tp = xsub(pow_f(xadd(xmul(0.249f, log_la), 0.65f), 2.7f), 0.72f);
        else tp = xsub(log_la, 1.255f);
        k.mp = xdiv(xsub(log_lda, 1.255f), tp);
        if (log_la <= -3.94f) ts = -2.86f;
        else if (log_la < -1.44f) ts = xsub(pow_f(xadd(xmul(0.405f, log_la), 1.6f), 2.18f), 2.86f);
        else ts = xsub(log_la, 0.395f);
        k.ms = xdiv(xsub(log_lda, 1.255f), ts);
        if (log_la < -2.0f) k.k = 1.0f;
        else if (log_la < 1.0f) k.k = xsub(1.0f, xmul(xadd(log_la, 2.0f), 1.0f / 3.0f));
        else k.k = 0.0f;
        break;
    }
    default:
        k.sf = 1.0f / 683.0f;
        break;
    }
    acc->s = k;
    acc->gmin = 0xffffffffu;
    acc->gmax = 0u;
}

// Coarse records: per group of kCoarse chunks and candidate binade, the
// sums of its chunks' records.
constexpr int kCoarse = 8;

__global__ void k_tone_coarse(const ChunkSum *__restrict__ rec, int64_t nchunks, int64_t ncoarse,
                              ChunkSum *__restrict__ crec)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncoarse * 32) return;
    const int64_t c = idx >> 5;
    const int ei = (int)(idx & 31);
    long long pos = 0, neg = 0;
    int32_t tie = 0;
    for (int f = 0; f < kCoarse; ++f) {
        const int64_t j = c * kCoarse + f;
        if (j >= nchunks) break;
        const ChunkSum r = rec[j * 32 + ei];
        pos += r.pos;
        neg += r.neg;
        tie |= r.tie;
    }
    ChunkSum sum;
    sum.pos = sat32(pos);
    sum.neg = sat32(neg);
    sum.tie = tie;
    sum.pad = 0;
    crec[idx] = sum;
}

// S as e and M (S = M * 2^(e-23), 2^23 <= |M| < 2^24) for a normal S, and
// back for 2^23 < |M| < 2^24: integer operations on the bits only.
__device__ __forceinline__ bool split(float S, int &e, int32_t &M)
{
    const uint32_t b = __float_as_uint(S);
    const uint32_t ex = (b >> 23) & 0xffu;
    if (ex == 0u || ex == 0xffu) return false;   // zero, subnormal, infinite
    e = (int)ex - 127;
    const int32_t m = (int32_t)((b & 0x7fffffu) | 0x800000u);
    M = (b >> 31) ? -m : m;
    return true;
}
__device__ __forceinline__ float join(int e, int32_t M)
{
    const uint32_t sign = (M < 0) ? 0x80000000u : 0u;
    const uint32_t m = (uint32_t)((M < 0) ? -M : M);
    return __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | (m & 0x7fffffu));
}

// Whether M + P stays strictly inside the binade of M (units of u): then
// the exact partial sum lies inside it too and rounds on the grid of u.
__device__ __forceinline__ bool inside(int32_t M, int32_t P)
{
    const int32_t lo = (1 << 23) + 1, hi = (1 << 24) - 1;
    const int32_t v = M + P;
    return (M > 0) ? (v >= lo && v <= hi) : (v <= -lo && v >= -hi);
}

// Records first .. first + 31 (lane l: record first + l, for the binade of
// S; count valid) tried as one run: each record keeps S in its binade when
// M + (the increments of the records before it) + its neg and + its pos
// both stay inside and it has no tie.  The records before the first that
// fails are applied (exactly: every prefix sum stays on the grid of u).
// Returns how many were applied; 32 when all were.  Uniform across the warp.
__device__ __forceinline__ int apply_records(float &S, const ChunkSum *__restrict__ recs, int64_t first, int64_t count,
                                             int64_t stride, int32_t e_lo)
{
    const int lane = threadIdx.x & 31;
    int e;
    int32_t M;
    if (!split(S, e, M) || e - e_lo < 0 || e - e_lo >= 32) return 0;
    const int64_t idx = first + lane;
    ChunkSum r = {0, 0, 1, 0};
    if (idx < count) r = recs[idx * stride + (e - e_lo)];
    // this record's total, clamped: a record beyond +-2^24 never applies
    const int32_t d = min(max(r.pos + r.neg, -(1 << 25)), 1 << 25);
    int32_t incl = d;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const int32_t base = incl - d;
    const bool ok = idx < count && !r.tie && inside(M, base + r.neg) && inside(M, base + r.pos);
    const uint32_t fail = __ballot_sync(0xffffffffu, !ok);
    const int n = fail ? __ffs(fail) - 1 : 32;
    if (n > 0) S = join(e, M + __shfl_sync(0xffffffffu, incl, n - 1));
    return n;
}

// Adds slice v (32 terms, lane order) to S term by term.
__device__ __forceinline__ float add_slice(float S, float v)
{
#pragma unroll
    for (int l = 0; l < 32; ++l) S = xadd(S, __shfl_sync(0xffffffffu, v, l));
    return S;
}

// The 512 terms of chunk j (16 slices of 32, slice q holding terms
// q*32 .. q*32+31 in lane order) added to S in order.  For S's binade all
// remaining slices are scanned at once (rounded increments, warp scans,
// running bases); the slices before the first one whose prefix sums leave
// the binade (or hold a tie) are applied in one step, that slice term by
// term, and the rest tried again in the new binade.  Uniform across the warp.
__device__ float sum_chunk(float S, const float *__restrict__ terms, int64_t j)
{
    constexpr int Q = kSumChunk / 32;
    const int lane = threadIdx.x & 31;
    float a[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) a[q] = terms[j * kSumChunk + q * 32 + lane];
    int q0 = 0;
    for (int round = 0; round <= Q && q0 < Q; ++round) {
        int e;
        int32_t M;
        int bad = q0;   // the first slice that cannot be applied
        if (split(S, e, M) && 23 - e <= 127) {
            const float scale = __int_as_float((23 - e + 127) << 23);   // 2^(23-e)
            int32_t P[Q];
            uint32_t fails = 0;   // bit q: slice q fails in this lane
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const float k = xmul(a[q], scale);   // exact: a power-of-two scale
                const bool big = !(fabsf(k) < 33554432.0f);
                const bool tie = !big && xsub(k, floorf(k)) == 0.5f;
                P[q] = big ? 0 : __float2int_rn(k);
                if (big || tie) fails |= 1u << q;
            }
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const int32_t v = __shfl_up_sync(0xffffffffu, P[q], o);
                    if (lane >= o) P[q] += v;
                }
            // running base over the slices from q0 on
            int32_t base = 0;
            int32_t base_at[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                base_at[q] = base;
                if (q >= q0) base += min(max(__shfl_sync(0xffffffffu, P[q], 31), -(1 << 25)), 1 << 25);
            }
#pragma unroll
            for (int q = 0; q < Q; ++q)
                if (q >= q0 && !inside(M, base_at[q] + P[q])) fails |= 1u << q;
            fails = __reduce_or_sync(0xffffffffu, fails) & ~((1u << q0) - 1u);
            bad = fails ? __ffs(fails) - 1 : Q;
            if (bad > q0) {
                int32_t upto = 0;
#pragma unroll
                for (int q = 0; q < Q; ++q)
                    if (q == bad - 1) upto = __shfl_sync(0xffffffffu, base_at[q] + P[q], 31);
                S = join(e, M + upto);
            }
        }
        if (bad >= Q) break;
        float v = 0.0f;
#pragma unroll
        for (int q = 0; q < Q; ++q)
            if (q == bad) v = a[q];
        S = add_slice(S, v);
        q0 = bad + 1;
    }
    return S;
}

// One warp walks the groups of kCoarse chunks in order, 32 group records at
// a time (apply_records); a group that cannot be applied goes chunk by
// chunk (its records), a chunk slice by slice (sum_chunk).  Then the scale
// factors.
__global__ void __launch_bounds__(32) k_tone_sum(const float *__restrict__ terms, const ChunkSum *__restrict__ rec,
                                                 const ChunkSum *__restrict__ crec, int64_t nchunks, int64_t ncoarse,
                                                 int32_t e_lo, ToneView t, ToneAcc *acc, bool scalars)
{
    float S = 0.0f;
    int64_t c = 0;
    for (int64_t guard = 0; c < ncoarse && guard < 4 * ncoarse + 64; ++guard) {
        const int n = apply_records(S, crec, c, ncoarse, 32, e_lo);
        c += n;
        if (n == 32 || c >= ncoarse) continue;
        // group c chunk by chunk
        const int64_t j_end = (c + 1) * kCoarse < nchunks ? (c + 1) * kCoarse : nchunks;
        int64_t j = c * kCoarse;
        for (int g2 = 0; j < j_end && g2 <= kCoarse; ++g2) {
            const int m = apply_records(S, rec, j, j_end, 32, e_lo);
            j += m;
            if (j >= j_end) break;
            S = sum_chunk(S, terms, j);
            ++j;
        }
        ++c;
    }
    if (threadIdx.x == 0) {
        acc->sum_f = S;
        if (scalars) tone_scalars(t, acc);
    }
}

// Largest |value| (bit pattern of the magnitude; finite values order as
// their bits).
__global__ void k_abs_max(const float *__restrict__ v, int64_t n, uint32_t *out)
{
    uint32_t m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, __float_as_uint(v[i]) & 0x7fffffffu);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void __launch_bounds__(kToneThreads) k_tone_range(const float *__restrict__ fimg, int64_t n, ToneView t,
                                                             ToneAcc *acc)
{
    const ToneScalars k = acc->s;
    uint32_t lo = 0xffffffffu, hi = 0u;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const Yxy p = to_yxy<true>(make_float3(fimg[3 * i], fimg[3 * i + 1], fimg[3 * i + 2]), t);
        const uint32_t key =
            order_key((t.mode == RT_TONE_GLOBAL_BILATERAL) ? t.bil[i] : map_lum<true>(p.Y, t, k, acc->h));
        lo = min(lo, key);
        hi = max(hi, key);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&acc->gmin, lo);
        atomicMax(&acc->gmax, hi);
    }
}

// One output pixel: each of its aa_x * aa_y samples through the chain, then
// clip_image_to_rgb's sum (a_x outer, a_y inner) and division.  inexact
// (nullable) is set when a single-precision library call took part: every
// mode's luminance map but the bilateral one (precomputed exactly), or a
// gamma power inside (0, 1).
template <bool EXACT>
__device__ __forceinline__ float3 tone_pixel(const float *__restrict__ fimg, int32_t fw, int32_t aa_x, int32_t aa_y,
                                             int32_t ox, int32_t oy, const ToneView &t, const ToneScalars &k,
                                             const ToneHist &hh, bool stretch, float offset, float scale,
                                             float samples, bool *inexact = nullptr)
{
    if (inexact) *inexact = t.enabled && t.mode != RT_TONE_GLOBAL_BILATERAL;
    float3 a = make_float3(0.0f, 0.0f, 0.0f);
    for (int32_t ax = 0; ax < aa_x; ++ax)
        for (int32_t ay = 0; ay < aa_y; ++ay) {
            const int64_t s = (int64_t)(ox * aa_x + ax) + (int64_t)(oy * aa_y + ay) * fw;
            float3 c = make_float3(fimg[3 * s], fimg[3 * s + 1], fimg[3 * s + 2]);
            if (t.enabled) {
                const Yxy p = to_yxy<EXACT>(c, t);
                float g = (t.mode == RT_TONE_GLOBAL_BILATERAL) ? t.bil[s] : map_lum<EXACT>(p.Y, t, k, hh);
                if (stretch) g = xmul(xadd(g, offset), scale);
                c = to_rgb<EXACT>(p.x, g, p.y, t.gamma, inexact);
            }
            a = xadd3(a, c);
        }
    return make_float3(xdiv(a.x, samples), xdiv(a.y, samples), xdiv(a.z, samples));
}

// A channel within kTruncGuard of an integer in [0, 255] may truncate
// differently once its float library calls are exact.
__device__ __forceinline__ bool near_integer(float v)
{
    return v > -kTruncGuard && v < 255.0f + kTruncGuard && fabsf(v - rintf(v)) < kTruncGuard;
}

// The stretch parameters of camera.cc:1428-1450: applied when the mapped
// range is positive or negative and not a single value.
struct Stretch {
    bool on;
    float offset, scale;
};
__device__ __forceinline__ Stretch stretch_of(const ToneView &t, const ToneAcc *acc)
{
    Stretch r = {false, 0.0f, 1.0f};
    if (!t.enabled || !t.stretch) return r;
    const float minY2 = key_float(acc->gmin), maxY2 = key_float(acc->gmax);
    if (((minY2 > 0.0f) || (maxY2 < 0.0f)) && (minY2 < maxY2)) {
        r.on = true;
        r.offset = (0.0f < -minY2) ? 0.0f : -minY2;          // std::min(-minY2, 0)
        const float top = (maxY2 < 1.0f) ? maxY2 : 1.0f;     // std::min(1, maxY2)
        const float bot = (0.0f < minY2) ? minY2 : 0.0f;     // std::max(0, minY2)
        r.scale = xdiv(1.0f, xsub(top, bot));
    }
    return r;
}

__device__ __forceinline__ void store_pixel(uint8_t *rgb, int64_t o, float3 v)
{
    rgb[3 * o] = clip8(v.x);
    rgb[3 * o + 1] = clip8(v.y);
    rgb[3 * o + 2] = clip8(v.z);
}

// Per output pixel: tone_pixel with the single-precision library calls; a
// pixel with a channel near a truncation boundary is queued for k_tone_fix
// instead (warp-aggregated append), then the clamp and truncation of
// clip_image_to_rgb.
__global__ void __launch_bounds__(kToneThreads) k_tone_final(const float *__restrict__ fimg, int32_t fw, int32_t aa_x,
                                                             int32_t aa_y, int32_t ow, int32_t oh, ToneView t,
                                                             ToneAcc *acc, int32_t *__restrict__ redo,
                                                             uint8_t *__restrict__ rgb)
{
    ToneScalars k = {};
    if (t.enabled) k = acc->s;
    const Stretch sr = stretch_of(t, acc);
    const int64_t npix = (int64_t)ow * oh;
    const float samples = (float)(aa_x * aa_y);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t steps = (npix + stride - 1) / stride;   // uniform trip count: whole warps append
    for (int64_t it = 0; it < steps; ++it) {
        const int64_t o = start + it * stride;
        bool queue = false;
        if (o < npix) {
            const int32_t oy = (int32_t)(o / ow), ox = (int32_t)(o - (int64_t)oy * ow);
            bool inexact = false;
            const float3 v = tone_pixel<false>(fimg, fw, aa_x, aa_y, ox, oy, t, k, acc->h, sr.on, sr.offset, sr.scale,
                                               samples, &inexact);
            queue = inexact && (near_integer(v.x) || near_integer(v.y) || near_integer(v.z));
            if (!queue) store_pixel(rgb, o, v);
        }
        const uint32_t b = __ballot_sync(0xffffffffu, queue);
        if (b) {
            int base = 0;
            const int lane = threadIdx.x & 31;
            if (lane == 0) base = atomicAdd(&acc->redo, __popc(b));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (queue) redo[base + __popc(b & ((1u << lane) - 1u))] = (int32_t)o;
        }
    }
}

// The queued pixels, with the library calls evaluated exactly.
__global__ void __launch_bounds__(kToneThreads) k_tone_fix(const float *__restrict__ fimg, int32_t fw, int32_t aa_x,
                                                           int32_t aa_y, int32_t ow, ToneView t, const ToneAcc *acc,
                                                           const int32_t *__restrict__ redo, uint8_t *__restrict__ rgb)
{
    const ToneScalars k = acc->s;
    const Stretch sr = stretch_of(t, acc);
    const int n = acc->redo;
    const float samples = (float)(aa_x * aa_y);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int64_t o = redo[i];
        const int32_t oy = (int32_t)(o / ow), ox = (int32_t)(o - (int64_t)oy * ow);
        store_pixel(rgb, o,
                    tone_pixel<true>(fimg, fw, aa_x, aa_y, ox, oy, t, k, acc->h, sr.on, sr.offset, sr.scale, samples));
    }
}

// ---- camera::bilateral_filter_tone_map(0.4, s, 0.4, s), s = 0.02 min(w, h)
// (camera.cc:1354-1358, 1632-1812)
//
// The bilateral grid of log10 luminance: one cell per s samples each way and
// per 0.4 decades, 3 cells of padding (sigma = 1 cell: 2 * 1 + 1).  The
// reference blurs it with a Gaussian through single-precision FFTW plans of
// dims (W, H, D) over its x-fastest array (index x + W (y + H z)), FFTW's
// last dimension varying fastest: the circular convolution runs over those
// axes of the flat array.  Here the same convolution is computed exactly, as
// discrete Fourier transforms along the three axes in double.  Grid depth D
// depends on the frame's log-luminance range, so the kernels read the grid's
// size from BilState; the host sizes the scratch for the deepest grid a
// float's range allows.
constexpr int32_t kBilMaxDepth = 119;     // (log10 FLT_MAX - log10 3.18e-7) / 0.4 + 1 + 6
constexpr int32_t kBilMaxAxis = 4096;

struct BilState {
    uint32_t kmin, kmax;    // range of the log-luminance above the floor (order keys)
    uint32_t rmin, rmax;    // range of the sliced base (order keys)
    int32_t W, H, D;
    float in_min;
    int32_t err;
};

struct BilGeom {            // what the frame size fixes
    int32_t fw, fh;
    float s_sa;             // cells per sample: 0.02 * min(fw, fh)
    int32_t W, H;           // grid width and height (padding included)
};

__host__ __device__ inline BilGeom bil_geom(int32_t fw, int32_t fh)
{
    BilGeom g;
    g.fw = fw;
    g.fh = fh;
    g.s_sa = 0.02f * (float)(fw < fh ? fw : fh);
    g.W = (int32_t)((float)(fw - 1) / g.s_sa) + 1 + 6;
    g.H = (int32_t)((float)(fh - 1) / g.s_sa) + 1 + 6;
    return g;
}

// Log10 luminance of every sample (0 at or below the floor) and the range
// of those above it.
__global__ void __launch_bounds__(kToneThreads) k_bil_log(const float *__restrict__ fimg, int64_t n, ToneView t,
                                                          float *__restrict__ logi, BilState *bs)
{
    uint32_t lo = 0xffffffffu, hi = 0u;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const Yxy p = to_yxy<true>(make_float3(fimg[3 * i], fimg[3 * i + 1], fimg[3 * i + 2]), t);
        float l = 0.0f;
        if (p.Y > 3.18e-7f) {
            if (!log10_ff(p.Y, l)) l = log10_f(p.Y);   // correctly rounded either way
            const uint32_t k = order_key(l);
            lo = min(lo, k);
            hi = max(hi, k);
        }
        logi[i] = l;
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&bs->kmin, lo);
        atomicMax(&bs->kmax, hi);
    }
}

// The grid's depth from the range, and the twiddle factors of each axis
// (dims in FFTW's order: W slowest, D fastest).
__global__ void k_bil_dims(BilGeom g, BilState *bs, double *__restrict__ tw)
{
    __shared__ int32_t dims[3];
    if (threadIdx.x == 0) {
        bs->W = g.W;
        bs->H = g.H;
        int32_t D = 7;
        float in_min = 0.0f;
        if (bs->kmin <= bs->kmax) {
            in_min = key_float(bs->kmin);
            const float delta = xsub(key_float(bs->kmax), in_min);
            D = (int32_t)xdiv(delta, 0.4f) + 1 + 6;
        } else {
            bs->err = 1;   // no sample above the floor: the reference's range is undefined
        }
        if (D > kBilMaxDepth) { D = kBilMaxDepth; bs->err = 1; }
        bs->D = D;
        bs->in_min = in_min;
        dims[0] = g.W;
        dims[1] = g.H;
        dims[2] = D;
    }
    __syncthreads();
    for (int a = 0; a < 3; ++a) {
        const int32_t m = dims[a];
        for (int32_t k = threadIdx.x; k < m; k += blockDim.x) {
            double s, c;
            sincospi(2.0 * (double)k / (double)m, &s, &c);
            tw[2 * ((size_t)a * kBilMaxAxis + (size_t)k)] = c;
            tw[2 * ((size_t)a * kBilMaxAxis + (size_t)k) + 1] = s;
        }
    }
}

// The splat: count and log-luminance sum per cell (sums in double).  A
// cell spans about (0.02 min(w, h))^2 samples, so neighbouring lanes mostly
// share one: each run of lanes with the same cell sums first (one atomic
// per run).
// The cell of a sample outside the grid's depth (a floor sample's 0 beyond
// the range) is clamped into it.
__global__ void __launch_bounds__(kToneThreads) k_bil_splat(const float *__restrict__ logi, BilGeom g,
                                                            const BilState *bs, double *__restrict__ cnt,
                                                            double *__restrict__ sum)
{
    const int32_t W = bs->W, H = bs->H, D = bs->D;
    const float in_min = bs->in_min;
    const int64_t n = (int64_t)g.fw * g.fh;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t steps = (n + stride - 1) / stride;   // uniform trip count: whole warps match
    const int lane = threadIdx.x & 31;
    for (int64_t it = 0; it < steps; ++it) {
        const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x + it * stride;
        int64_t c = -1;
        double l = 0.0;
        if (i < n) {
            const int32_t y = (int32_t)(i / g.fw), x = (int32_t)(i - (int64_t)y * g.fw);
            const int32_t sx = (int32_t)xadd(xdiv((float)x, g.s_sa), 0.5f) + 3;
            const int32_t sy = (int32_t)xadd(xdiv((float)y, g.s_sa), 0.5f) + 3;
            int32_t sz = (int32_t)xadd(xdiv(xsub(logi[i], in_min), 0.4f), 0.5f) + 3;
            sz = sz < 0 ? 0 : (sz > D - 1 ? D - 1 : sz);
            if (sx >= 0 && sx < W && sy >= 0 && sy < H)   // always: the grid spans the frame
                c = (int64_t)sx + (int64_t)W * ((int64_t)sy + (int64_t)H * (int64_t)sz);
            l = (double)logi[i];
        }
        // runs of equal cells over consecutive lanes: each run's first lane
        // sums it (segmented tree reduction) and adds it to the cell
        const int64_t prev = __shfl_up_sync(0xffffffffu, c, 1);
        const uint32_t heads = __ballot_sync(0xffffffffu, lane == 0 || prev != c);
        const int run = __popc(heads & ((2u << lane) - 1u));
        double gc = (c >= 0) ? 1.0 : 0.0, gs = l;
        for (int o = 1; o < 32; o <<= 1) {
            const double vc = __shfl_down_sync(0xffffffffu, gc, o), vs = __shfl_down_sync(0xffffffffu, gs, o);
            const int r = __shfl_down_sync(0xffffffffu, run, o);
            if (lane + o < 32 && r == run) {
                gc += vc;
                gs += vs;
            }
        }
        if (((heads >> lane) & 1u) && c >= 0) {
            atomicAdd(cnt + c, gc);
            atomicAdd(sum + c, gs);
        }
    }
}

// The Gaussian of one cell with the reference's wrap-around coordinates,
// in binary32 (camera.cc:1678-1697).
__global__ void __launch_bounds__(kToneThreads) k_bil_kernel(const BilState *bs, double *__restrict__ kre,
                                                             double *__restrict__ kim)
{
    const int32_t W = bs->W, H = bs->H, D = bs->D;
    const int64_t N = (int64_t)W * H * D;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t x = (int32_t)(i % W), y = (int32_t)((i / W) % H), z = (int32_t)(i / ((int64_t)W * H));
        const float X = xsub((float)x, (x > (W >> 1)) ? (float)W : 0.0f);
        const float Y = xsub((float)y, (y > (H >> 1)) ? (float)H : 0.0f);
        const float Z = xsub((float)z, (z > (D >> 1)) ? (float)D : 0.0f);
        const float rr = xadd(xdiv(xadd(xmul(X, X), xmul(Y, Y)), 1.0f), xdiv(xmul(Z, Z), 1.0f));
        kre[i] = (double)exp_f(xmul(-rr, 0.5f));
        kim[i] = 0.0;
    }
}

// One discrete Fourier transform (sign -1 forward, +1 backward, not
// normalised) along axis a of nch complex channels (channel c at offset
// c * cstride) of dims (W, H, D), row-major with D fastest.
__global__ void __launch_bounds__(kToneThreads) k_bil_dft(const double *__restrict__ ire, const double *__restrict__ iim,
                                                          double *__restrict__ ore, double *__restrict__ oim,
                                                          const BilState *bs, const double *__restrict__ tw, int a,
                                                          double sign, int nch, int64_t cstride)
{
    const int32_t W = bs->W, H = bs->H, D = bs->D;
    const int64_t N = (int64_t)W * H * D;
    const int32_t m = a == 0 ? W : (a == 1 ? H : D);
    const int64_t stride = a == 0 ? (int64_t)H * D : (a == 1 ? (int64_t)D : 1);
    const double *twa = tw + 2 * (size_t)a * kBilMaxAxis;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < (int64_t)nch * N;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = g / N, i = g - c * N;
        const int32_t k = (int32_t)((i / stride) % m);
        const int64_t base = c * cstride + i - (int64_t)k * stride;
        double sr = 0.0, si = 0.0;
        int32_t t = 0;   // j * k mod m
        for (int32_t j = 0; j < m; ++j) {
            const double vr = ire[base + (int64_t)j * stride], vi = iim[base + (int64_t)j * stride];
            const double cr = twa[2 * t], ci = sign * twa[2 * t + 1];
            sr = fma(vr, cr, fma(-vi, ci, sr));
            si = fma(vr, ci, fma(vi, cr, si));
            t += k;
            if (t >= m) t -= m;
        }
        ore[c * cstride + i] = sr;
        oim[c * cstride + i] = si;
    }
}

// The product of the channels' spectra with the kernel's, over N (the
// inverse transform is not normalised).
__global__ void __launch_bounds__(kToneThreads) k_bil_mul(const double *__restrict__ are, const double *__restrict__ aim,
                                                          const double *__restrict__ kre,
                                                          const double *__restrict__ kim, double *__restrict__ ore,
                                                          double *__restrict__ oim, const BilState *bs, int64_t cstride)
{
    const int64_t N = (int64_t)bs->W * bs->H * bs->D;
    const double inv = 1.0 / (double)N;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < 2 * N; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = g / N, i = g - c * N;
        const double ar = are[c * cstride + i], ai = aim[c * cstride + i];
        ore[c * cstride + i] = (ar * kre[i] - ai * kim[i]) * inv;
        oim[c * cstride + i] = (ar * kim[i] + ai * kre[i]) * inv;
    }
}

// The trilinear slice of the blurred grid at every sample (camera.cc:
// 1740-1789, binary32 in the reference's order on the grid rounded to
// binary32) and the range of the result.
__global__ void __launch_bounds__(kToneThreads) k_bil_slice(const float *__restrict__ logi, BilGeom g,
                                                            BilState *bs, const double *__restrict__ blur,
                                                            int64_t cstride, float *__restrict__ res)
{
    const int32_t W = bs->W, H = bs->H, D = bs->D;
    const float in_min = bs->in_min;
    const int64_t n = (int64_t)g.fw * g.fh;
    const double *bw = blur, *biw = blur + cstride;
    uint32_t lo = 0xffffffffu, hi = 0u;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t y = (int32_t)(i / g.fw), x = (int32_t)(i - (int64_t)y * g.fw);
        const float z = xsub(logi[i], in_min);
        const float xa_ = xadd(xdiv((float)x, g.s_sa), 3.0f);
        const float ya_ = xadd(xdiv((float)y, g.s_sa), 3.0f);
        const float za_ = xadd(xdiv(z, 0.4f), 3.0f);
        const int32_t xi = max(0, min((int32_t)xa_, W - 1)), xx = max(0, min(xi + 1, W - 1));
        const int32_t yi = max(0, min((int32_t)ya_, H - 1)), yy = max(0, min(yi + 1, H - 1));
        const int32_t zi = max(0, min((int32_t)za_, D - 1)), zz = max(0, min(zi + 1, D - 1));
        const float ax = xsub(xa_, (float)xi), ay = xsub(ya_, (float)yi), az = xsub(za_, (float)zi);
        const float bx = xsub(1.0f, ax), by = xsub(1.0f, ay), bz = xsub(1.0f, az);
        auto at = [&](const double *a, int32_t X, int32_t Y, int32_t Z) {
            return (float)a[(size_t)X + (size_t)W * ((size_t)Y + (size_t)H * (size_t)Z)];
        };
        auto tri = [&](const double *a) {
            float s = xmul(xmul(xmul(bx, by), bz), at(a, xi, yi, zi));
            s = xadd(s, xmul(xmul(xmul(ax, by), bz), at(a, xx, yi, zi)));
            s = xadd(s, xmul(xmul(xmul(bx, ay), bz), at(a, xi, yy, zi)));
            s = xadd(s, xmul(xmul(xmul(ax, ay), bz), at(a, xx, yy, zi)));
            s = xadd(s, xmul(xmul(xmul(bx, by), az), at(a, xi, yi, zz)));
            s = xadd(s, xmul(xmul(xmul(ax, by), az), at(a, xx, yi, zz)));
            s = xadd(s, xmul(xmul(xmul(bx, ay), az), at(a, xi, yy, zz)));
            s = xadd(s, xmul(xmul(xmul(ax, ay), az), at(a, xx, yy, zz)));
            return s;
        };
        const float r = xdiv(tri(biw), tri(bw));
        res[i] = r;
        const uint32_t k = order_key(r);
        lo = min(lo, k);
        hi = max(hi, k);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&bs->rmin, lo);
        atomicMax(&bs->rmax, hi);
    }
}

// The contrast compression (camera.cc:1793-1800): Y = 10^(base * gamma +
// detail) / 255, gamma = log10(300) / (base range).
__global__ void __launch_bounds__(kToneThreads) k_bil_scale(const float *__restrict__ logi,
                                                            const float *__restrict__ res, int64_t n,
                                                            const BilState *bs, float *__restrict__ bil)
{
    const float gamma = xdiv(log10_f(300.0f), xsub(key_float(bs->rmax), key_float(bs->rmin)));
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float r = res[i];
        // powf(10, e) as 2^(e log2 10) in double, rounded once: the
        // product's relative error (2^-53) is far below a float's ulp
        const float e = xadd(xmul(r, gamma), xsub(logi[i], r));
        const float scaled = (float)exp2((double)e * 3.321928094887362347870319429489);
        bil[i] = xmul(scaled, 1.0f / 255.0f);
    }
}

int blocks_for(int64_t n, int sm_count)
{
    const int64_t b = (n + kToneThreads - 1) / kToneThreads;
    const int64_t cap = (int64_t)sm_count * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

size_t tone_scratch_bytes(int64_t n, int64_t blocks)
{
    const int64_t nchunks = (n + kSumChunk - 1) / kSumChunk;
    const int64_t ncoarse = (nchunks + kCoarse - 1) / kCoarse;
    return (size_t)nchunks * kSumChunk * sizeof(float) + (size_t)(nchunks + ncoarse) * 32 * sizeof(ChunkSum) +
           (size_t)n * sizeof(int32_t) +   // redo queue (at most one entry per output pixel)
           (size_t)blocks * sizeof(float) +  // histogram modes: the per-degree luminance blocks
           (size_t)2 * 2 * 4096 * sizeof(float);   // and their bounds (at most 4096 per axis)
}

bool bilateral_grid_fits(int32_t fw, int32_t fh)
{
    const BilGeom g = bil_geom(fw, fh);
    return g.W <= kBilMaxAxis && g.H <= kBilMaxAxis && (int64_t)g.W * g.H * kBilMaxDepth <= ((int64_t)1 << 26);
}

size_t bilateral_scratch_bytes(int32_t fw, int32_t fh)
{
    const BilGeom g = bil_geom(fw, fh);
    const size_t nmax = (size_t)g.W * (size_t)g.H * (size_t)kBilMaxDepth;
    const size_t n = (size_t)fw * (size_t)fh;
    // 256-byte alignment of the start and of the doubles
    return 3 * 256 + 3 * n * sizeof(float) + 12 * nmax * sizeof(double) + 6 * (size_t)kBilMaxAxis * sizeof(double);
}

static char *align256(char *p) { return (char *)(((uintptr_t)p + 255u) & ~(uintptr_t)255u); }

// The bilateral mode's per-sample luminance into scratch (layout: state |
// log | base | mapped | kernel re, im | temp re, im | A re, im (2 channels)
// | B re, im (2 channels) | twiddles); returns the mapped array.
static const float *launch_bilateral(const float *fimg, int32_t fw, int32_t fh, const ToneView &t, void *scratch,
                                     int sm_count, cudaStream_t st)
{
    const BilGeom g = bil_geom(fw, fh);
    const int64_t n = (int64_t)fw * fh;
    const int64_t nmax = (int64_t)g.W * g.H * kBilMaxDepth;
    char *p = align256((char *)scratch);
    BilState *bs = (BilState *)p;
    p += 256;
    float *logi = (float *)p;
    float *res = logi + n;
    float *bil = res + n;
    double *kre = (double *)align256((char *)(bil + n));
    double *kim = kre + nmax, *tre = kim + nmax, *tim = tre + nmax;
    double *are = tim + nmax, *aim = are + 2 * nmax, *bre = aim + 2 * nmax, *bim = bre + 2 * nmax;
    double *tw = bim + 2 * nmax;
    const BilState init = {0xffffffffu, 0u, 0xffffffffu, 0u, 0, 0, 0, 0.0f, 0};
    cudaMemcpyAsync(bs, &init, sizeof(init), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(are, 0, 4 * (size_t)nmax * sizeof(double), st);   // A re and im, both channels
    const int bn = blocks_for(n, sm_count), bg = blocks_for(2 * nmax, sm_count);
    k_bil_log<<<bn, kToneThreads, 0, st>>>(fimg, n, t, logi, bs);
    k_bil_dims<<<1, 256, 0, st>>>(g, bs, tw);
    k_bil_splat<<<bn, kToneThreads, 0, st>>>(logi, g, bs, are, are + nmax);
    k_bil_kernel<<<bg, kToneThreads, 0, st>>>(bs, kre, kim);
    // kernel spectrum: K -> T -> K -> T
    k_bil_dft<<<bg, kToneThreads, 0, st>>>(kre, kim, tre, tim, bs, tw, 0, -1.0, 1, nmax);
    k_bil_dft<<<bg, kToneThreads, 0, st>>>(tre, tim, kre, kim, bs, tw, 1, -1.0, 1, nmax);
    k_bil_dft<<<bg, kToneThreads, 0, st>>>(kre, kim, tre, tim, bs, tw, 2, -1.0, 1, nmax);
    // the two channels' spectra: A -> B -> A -> B
    k_bil_dft<<<bg, kToneThreads, 0, st>>>(are, aim, bre, bim, bs, tw, 0, -1.0, 2, nmax);
    k_bil_dft<<<bg, kToneThreads, 0, st>>>(bre, bim, are, aim, bs, tw, 1, -1.0, 2, nmax);
    k_bil_dft<<<bg, kToneThreads, 0, st>>>(are, aim, bre, bim, bs, tw, 2, -1.0, 2, nmax);
    k_bil_mul<<<bg, kToneThreads, 0, st>>>(bre, bim, tre, tim, are, aim, bs, nmax);
    // back: A -> B -> A -> B
    k_bil_dft<<<bg, kToneThreads, 0, st>>>(are, aim, bre, bim, bs, tw, 0, +1.0, 2, nmax);
    k_bil_dft<<<bg, kToneThreads, 0, st>>>(bre, bim, are, aim, bs, tw, 1, +1.0, 2, nmax);
    k_bil_dft<<<bg, kToneThreads, 0, st>>>(are, aim, bre, bim, bs, tw, 2, +1.0, 2, nmax);
    k_bil_slice<<<bn, kToneThreads, 0, st>>>(logi, g, bs, bre, nmax, res);
    k_bil_scale<<<bn, kToneThreads, 0, st>>>(logi, res, n, bs, bil);
    return bil;
}

void launch_tone_map(const float *fimg, int32_t fw, int32_t fh, int32_t aa_x, int32_t aa_y, const ToneView &t_in,
                     uint8_t *rgb, ToneAcc *acc, void *scratch, int sm_count, cudaStream_t st)
{
    ToneView t = t_in;
    const int64_t n = (int64_t)fw * fh;
    const int32_t ow = fw / aa_x, oh = fh / aa_y;
    // scratch: terms | chunk records | coarse records | redo queue
    const int64_t nchunks = (n + kSumChunk - 1) / kSumChunk;
    const int64_t ncoarse = (nchunks + kCoarse - 1) / kCoarse;
    float *terms = (float *)scratch;
    ChunkSum *rec = (ChunkSum *)(terms + nchunks * kSumChunk);
    ChunkSum *crec = rec + nchunks * 32;
    int32_t *redo = (int32_t *)(crec + ncoarse * 32);
    float *hblocks = (float *)(redo + n);
    cudaMemsetAsync(acc, 0, sizeof(ToneAcc), st);
    // the stretch range starts empty (k_tone_sum sets it too, for the other modes)
    cudaMemsetAsync(&acc->gmin, 0xff, sizeof(uint32_t), st);
    if (t.enabled && t.mode == RT_TONE_GLOBAL_BILATERAL)
        t.bil = launch_bilateral(fimg, fw, fh, t, (char *)scratch + tone_scratch_bytes(n, 0), sm_count, st);
    if (t.enabled && t.mode != RT_TONE_GLOBAL_BILATERAL) {
        // candidate binades: |S| <= 39 n (|log10 Y| < 39 for any float Y)
        const int32_t e_hi = (int32_t)std::floor(std::log2(39.0 * (double)n)) + 1;
        const int32_t e_lo = e_hi - 31;
        k_tone_terms<<<(unsigned)nchunks, kSumThreads, 0, st>>>(fimg, nullptr, n, e_lo, terms, rec, acc);
        k_tone_coarse<<<(unsigned)((ncoarse * 32 + 255) / 256), 256, 0, st>>>(rec, nchunks, ncoarse, crec);
        k_tone_sum<<<1, 32, 0, st>>>(terms, rec, crec, nchunks, ncoarse, e_lo, t, acc, true);
        if (t.mode == RT_TONE_LOCAL_HISTOGRAM || t.mode == RT_TONE_LOCAL_HUMAN_HISTOGRAM) {
            const int64_t nb = (int64_t)t.hist_sx * t.hist_sy;
            float *bx = hblocks + nb, *by = bx + 2 * 4096;
            k_hist_bounds<<<1, 32, 0, st>>>(fw, fh, t, bx, by);
            k_hist_blocks<<<blocks_for(nb, sm_count), kToneThreads, 0, st>>>(fimg, fw, fh, t, bx, by, hblocks);
            k_hist_main<<<1, 128, 0, st>>>(hblocks, t, acc);
        }
    }
    if (t.enabled && t.stretch) k_tone_range<<<blocks_for(n, sm_count), kToneThreads, 0, st>>>(fimg, n, t, acc);
    k_tone_final<<<blocks_for((int64_t)ow * oh, sm_count), kToneThreads, 0, st>>>(fimg, fw, aa_x, aa_y, ow, oh, t, acc,
                                                                                  redo, rgb);
    if (t.enabled) k_tone_fix<<<sm_count, kToneThreads, 0, st>>>(fimg, fw, aa_x, aa_y, ow, t, acc, redo, rgb);
}

namespace {
// log10_ff against log10 in double on n floats spread over every binade
// (counter-based: element i maps to a float from its hash): out[0] counts
// disagreements of decided values, out[1] undecided values.
__global__ void k_check_log10(int64_t n, uint64_t seed, unsigned long long *out)
{
    unsigned long long bad = 0, undecided = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = (uint64_t)i * 0x9E3779B97F4A7C15ull + seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        // positive normal floats, with a quarter of them near 1 (where log10 is small)
        uint32_t bits = (uint32_t)(z & 0x7fffffffu);
        if ((z >> 62) == 0u) bits = 0x3f000000u + (uint32_t)((z >> 32) & 0x00ffffffu);
        if (bits < 0x00800000u || bits >= 0x7f800000u) continue;
        float r;
        if (log10_ff(__uint_as_float(bits), r)) {
            if (__float_as_uint(r) != __float_as_uint(log10_f(__uint_as_float(bits)))) ++bad;
        } else {
            ++undecided;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
        undecided += __shfl_xor_sync(0xffffffffu, undecided, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], bad);
        atomicAdd(&out[1], undecided);
    }
}
}  // namespace

void launch_check_log10(int64_t n, uint64_t seed, unsigned long long *out, int sm_count, cudaStream_t st)
{
    cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), st);
    k_check_log10<<<sm_count * 8, 256, 0, st>>>(n, seed, out);
}

void launch_abs_max(const float *v, int64_t n, uint32_t *out, int sm_count, cudaStream_t st)
{
    cudaMemsetAsync(out, 0, sizeof(uint32_t), st);
    k_abs_max<<<blocks_for(n, sm_count), kToneThreads, 0, st>>>(v, n, out);
}

void launch_sequential_sum(const float *v, int64_t n, float max_abs, ToneAcc *acc, void *scratch, int sm_count,
                           cudaStream_t st)
{
    (void)sm_count;
    const int64_t nchunks = (n + kSumChunk - 1) / kSumChunk;
    const int64_t ncoarse = (nchunks + kCoarse - 1) / kCoarse;
    float *terms = (float *)scratch;
    ChunkSum *rec = (ChunkSum *)(terms + nchunks * kSumChunk);
    ChunkSum *crec = rec + nchunks * 32;
    // candidate binades: |S| <= max_abs * n
    int32_t e_hi = (int32_t)std::floor(std::log2((double)max_abs * (double)n)) + 1;
    if (e_hi > 128) e_hi = 128;
    const int32_t e_lo = e_hi - 31;
    cudaMemsetAsync(acc, 0, sizeof(ToneAcc), st);
    ToneView t = {};
    k_tone_terms<<<(unsigned)nchunks, kSumThreads, 0, st>>>(nullptr, v, n, e_lo, terms, rec, acc);
    k_tone_coarse<<<(unsigned)((ncoarse * 32 + 255) / 256), 256, 0, st>>>(rec, nchunks, ncoarse, crec);
    k_tone_sum<<<1, 32, 0, st>>>(terms, rec, crec, nchunks, ncoarse, e_lo, t, acc, false);
}

}  // namespace rtc
