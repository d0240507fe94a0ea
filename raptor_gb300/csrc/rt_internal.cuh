// rt_internal.cuh -- device data layout and IEEE-exact arithmetic shared by
// the build, traversal and shading kernels of the GB300 ray-tracing core.
#pragma once

#include <cstdint>
#include <cfloat>
#include <cuda_runtime.h>

#include "../../include/rtcore.h"

namespace rtc {

// ---------------------------------------------------------------- limits
constexpr int kStackSize = 48;          // traversal stack entries (>= max tree depth)
constexpr int kMaxDepth = 40;           // build fails above this wide-tree depth
constexpr int kMaxSegments = 1024;   // scenes per batched build
constexpr int kMaxLeafTris = 3;         // triangles per leaf slot (unary count in 3 bits)
constexpr float kEpsilon = 1.0e-3f;     // common/common.cc:14
constexpr float kDetEps = 0.000001f;    // triangle.h:201
constexpr int kMaxTraversalSteps = 1 << 14;  // per-ray node-visit cap (status word on overflow)

// Device status bits (OR-ed into one word per launch).
constexpr uint32_t kStatusStackOverflow = 1u;
constexpr uint32_t kStatusStepLimit = 2u;
constexpr uint32_t kStatusBadIndex = 4u;   // a node/triangle index outside the scene (never expected)

// --------------------------------------------------------- data layout
// 8-wide node with 8-bit quantised child boxes: 80 bytes = 5 x 16 B, read
// with 128-bit loads.  Child box (axis k) = p_k + q * 2^(e_k - 127) where e
// is a biased float exponent; boxes are padded one grid unit outwards.
struct __align__(16) WideNode {
    float px, py, pz;         // quantisation origin
    uint8_t ex, ey, ez;       // biased exponents of the per-axis scale
    uint8_t imask;            // bit s set: slot s is an internal child
    uint32_t child_base;      // first child node (internal children contiguous, slot order)
    uint32_t tri_base;        // first packed triangle of this node's leaves
    uint8_t meta[8];          // per slot: 0 empty; internal 0x20|(24+s); leaf (unary<<5)|offset
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
    uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(WideNode) == 80, "wide node must be 80 bytes");

// Packed triangle in leaf order: vertices a, b, c (exactly the caller's, so
// neighbouring triangles share bit-identical edges), the caller's id and
// flags: 48 B.
struct __align__(16) PackedTri {
    float4 w0;   // a.x a.y a.z b.x
    float4 w1;   // b.y b.z c.x c.y
    float4 w2;   // c.z id(bits) flags(bits) 0
};

// Per-triangle shading record in the caller's order: face normal n
// (triangle.h:171-175) and vertex c (for hit refinement, triangle.h:466-470).
struct __align__(16) ShadeTri {
    float4 n_cx;   // n.x n.y n.z c.x
    float2 c_yz;   // c.y c.z
    float2 pad;
};

struct SceneView {
    const WideNode *nodes;
    const PackedTri *tris;
    const ShadeTri *shade;
    const int3 *idx;          // vertex indices per triangle (caller's order)
    const float *vattr;       // 3 floats per vertex or nullptr
    const uint32_t *flags;    // per triangle (caller's order)
    int32_t ntris;
    int32_t nnodes;
    int32_t root;             // root wide node of this scene
    int32_t tri_base;         // subtracted from packed ids to give the caller's ids
    int32_t isect;            // RT_ISECT_REFERENCE or RT_ISECT_WATERTIGHT
    const int32_t *mat = nullptr;   // material index per triangle (caller's order) or nullptr
    const float *cnorm = nullptr;   // 9 floats per triangle: corner normals a, b, c (x of a = FLT_MAX: none)
};

struct CameraView {
    float3 c, X, Y, Z;
    float x_m, y_m, x_inc, y_inc, t;
    int32_t xres, yres;
    float3 background;
};

struct LightView {
    int32_t kind;
    float3 rgb255;     // rgb / 255 (light.h:17-34 store rgb / 255.0f)
    float3 pos;
    float3 dir;
    float dist_sign;   // +-1e15 for directional lights (light.h:69-86)
    float d;
    float s_a, s_b;    // spot cone (s_b = 0: none)
    float radius;      // spherical light's radius (soft shadows only)
};

struct MaterialView {
    float3 ka, kd, ks;
    float ns;
    float rf;    // mirror reflectivity (0: none)
    float tran;  // transparency: refracted colour weight (0: opaque)
    float ri;    // refractive index
    uint32_t flags;   // RT_MAT_NO_VERTEX_COLOUR
};

// Materials of a frame (rt_render_materials), indexed per triangle by
// SceneView::mat.
struct MaterialTable {
    int32_t n;
    MaterialView m[RT_MAX_MATERIALS];
};

// -------------------------------------------------- IEEE-exact helpers
// Explicit round-to-nearest intrinsics are never contracted into FMAs, so
// these reproduce the reference's binary32 results bit for bit.
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }

__device__ __forceinline__ float3 xsub3(float3 a, float3 b) { return make_float3(xsub(a.x, b.x), xsub(a.y, b.y), xsub(a.z, b.z)); }
__device__ __forceinline__ float3 xadd3(float3 a, float3 b) { return make_float3(xadd(a.x, b.x), xadd(a.y, b.y), xadd(a.z, b.z)); }
__device__ __forceinline__ float3 xmul3(float3 a, float s) { return make_float3(xmul(a.x, s), xmul(a.y, s), xmul(a.z, s)); }
__device__ __forceinline__ float3 xdiv3(float3 a, float s) { return make_float3(xdiv(a.x, s), xdiv(a.y, s), xdiv(a.z, s)); }
// dot_product, left to right (common/point_t.h:522-525)
__device__ __forceinline__ float xdot(float3 a, float3 b) { return xadd(xadd(xmul(a.x, b.x), xmul(a.y, b.y)), xmul(a.z, b.z)); }
// cross_product (common/point_t.h:511-514)
__device__ __forceinline__ float3 xcross(float3 a, float3 b)
{
    return make_float3(xsub(xmul(a.y, b.z), xmul(a.z, b.y)), xsub(xmul(a.z, b.x), xmul(a.x, b.z)),
                       xsub(xmul(a.x, b.y), xmul(a.y, b.x)));
}
// magnitude (point_t.h:357) and normalise with sqrt + divide (point_t.h:571-585)
__device__ __forceinline__ float xmag(float3 a) { return __fsqrt_rn(xadd(xadd(xmul(a.x, a.x), xmul(a.y, a.y)), xmul(a.z, a.z))); }
__device__ __forceinline__ float3 xnorm(float3 a) { return xdiv3(a, xmag(a)); }
// std::min / std::max operand semantics
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }

// Host-side counterparts of the view structs are filled in rt_api.cu.

}  // namespace rtc
