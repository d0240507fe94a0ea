// rt_build.cuh -- interface of the GPU acceleration-structure builder.
#pragma once

#include "rt_internal.cuh"

namespace rtc {

enum : int32_t { kBuilderLbvh = 0, kBuilderPloc = 1, kBuilderHploc = 2 };

struct BuildInputs {
    int32_t ntris;
    const float *verts;       // device, 3 floats per vertex
    const int3 *idx;          // device, caller's order
    const uint32_t *flags;    // device or nullptr
    ShadeTri *shade;          // device out, ntris
    WideNode *nodes;          // device out, max_nodes
    PackedTri *tris;          // device out, ntris
    int32_t max_nodes;
    int32_t sm_count;
    int32_t *host_scratch;    // pinned host, >= 6 + kMaxDepth ints
    int32_t builder = kBuilderPloc;   // binary tree: kBuilderLbvh, kBuilderPloc or kBuilderHploc
    int32_t morton_bits = 0;          // bits per axis of the sort key (0: from ntris)
    // several scenes in one build (a batch): segment of each triangle and
    // the triangle offset of each segment (nseg + 1 entries, host or device).
    // nseg <= 1: a single scene, both may be nullptr.  Segment s's root is
    // wide node s.
    int32_t nseg = 1;
    const int32_t *seg_of_tri = nullptr;
    const int32_t *seg_first = nullptr;
};

// Device arrays a build leaves in its scratch so that the same tree can be
// refitted to moved vertices (single scenes only).
struct RefitArrays {
    bool valid = false;
    const int32_t *vals = nullptr;          // sorted position -> triangle id
    const int32_t *left = nullptr, *right = nullptr, *parent = nullptr, *leaf_parent = nullptr;
    float4 *blo = nullptr, *bhi = nullptr;  // triangle boxes, caller's order
    float4 *llo = nullptr, *lhi = nullptr;  // leaf boxes, sorted order
    float4 *ilo = nullptr, *ihi = nullptr;  // binary node boxes
    int32_t *flags = nullptr;               // refit arrival counters
    const int32_t *slot_ref = nullptr;      // 8 binary refs per wide node
    int32_t *err = nullptr;
    int32_t ntris = 0, nnodes = 0, tri_slots = 0;
};

struct BuildResult {
    int32_t status = -8;      // 0 ok, else an rt_status code
    int32_t nodes = 0;
    int32_t tri_slots = 0;
    int32_t depth = 0;
    RefitArrays refit;
};

// Device scratch needed by build_wide_bvh for n triangles.
size_t build_temp_bytes(int32_t n);

// Build on stream st; synchronises st once at the end (and, for PLOC,
// once per kPlocGroup clustering iterations).
BuildResult build_wide_bvh(const BuildInputs &in, void *temp, size_t temp_bytes, cudaStream_t st);

// Refit the tree of a previous build (arrays K, still in its scratch) to
// moved vertices: shading records, boxes bottom-up, every wide node
// re-quantised, packed triangles rewritten; topology kept.  0 or an
// rt_status code.  Synchronises st once.
int32_t refit_wide_bvh(const RefitArrays &K, const float *verts, const int3 *idx, ShadeTri *shade, WideNode *nodes,
                       PackedTri *tris, int32_t *host_scratch, cudaStream_t st);

}  // namespace rtc
