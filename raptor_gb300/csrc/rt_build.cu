// rt_build.cu -- GPU acceleration-structure build for the GB300 ray-tracing
// core: Morton codes -> radix sort -> binary tree -> surface-area-guided
// collapse into 8-wide nodes with 8-bit quantised child boxes (layout after
// Ylitie, Karras & Laine, HPG 2017), conservatively rounded outwards so that
// no hit is ever lost.  The binary tree is either the Morton radix tree
// (LBVH, Karras HPG 2012, + bottom-up refit) or, by default, bottom-up
// locally-ordered clustering over the Morton order (PLOC, Meister & Bittner,
// IEEE TVCG 2018), which merges mutual nearest neighbours by surface area
// and gives trees with ~15-20 % less internal surface area.
//
// Replaces bvh_builder::build (raytracer/spatial_sub_division/
// bvh_builder.cc:18-178).  The reference builds a 2-wide tree with Morton
// codes + approximate agglomerative clustering on the CPU; hits do not
// depend on the tree, so a different tree gives the same closest hits.
#include <cub/device/device_radix_sort.cuh>

#include <vector>

#include "rt_build.cuh"

namespace rtc {

namespace {

__device__ __forceinline__ int ord_of(float f)
{
    const int i = __float_as_int(f);
    return (i >= 0) ? i : (i ^ 0x7fffffff);
}
__device__ __forceinline__ float of_ord(int i) { return __int_as_float((i >= 0) ? i : (i ^ 0x7fffffff)); }

// Per triangle (caller's order): shading record (face normal exactly as
// triangle.h:171-175, vertex c), bounding box, centroid bounds.
// With several segments (scenes of a batch) the centroid bounds are kept per
// segment: cbounds[6 * s + k] (k < 3 minimum, k >= 3 maximum).
__global__ void k_prep(const float *__restrict__ verts, const int3 *__restrict__ idx, int32_t n,
                       const int32_t *__restrict__ seg, int32_t nseg, ShadeTri *__restrict__ shade,
                       float4 *__restrict__ blo, float4 *__restrict__ bhi, int *__restrict__ cbounds)
{
    __shared__ int s_min[3][32], s_max[3][32];
    float cmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int3 t = idx[i];
        const float3 a = make_float3(verts[3 * t.x], verts[3 * t.x + 1], verts[3 * t.x + 2]);
        const float3 b = make_float3(verts[3 * t.y], verts[3 * t.y + 1], verts[3 * t.y + 2]);
        const float3 c = make_float3(verts[3 * t.z], verts[3 * t.z + 1], verts[3 * t.z + 2]);
        const float3 nn = xnorm(xcross(xsub3(b, a), xsub3(c, a)));
        ShadeTri st;
        st.n_cx = make_float4(nn.x, nn.y, nn.z, c.x);
        st.c_yz = make_float2(c.y, c.z);
        st.pad = make_float2(0.f, 0.f);
        shade[i] = st;
        const float3 lo = make_float3(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)));
        const float3 hi = make_float3(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)));
        blo[i] = make_float4(lo.x, lo.y, lo.z, 0.f);
        bhi[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
        const float cc[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
        if (nseg > 1) {
            // lanes of the same segment (usually the whole warp: a segment's
            // triangles are contiguous) reduce together; one atomic per group
            const int si = seg[i];
            const unsigned grp = __match_any_sync(__activemask(), si);
            const bool leader = (int)(threadIdx.x & 31) == __ffs(grp) - 1;
            int *cb = cbounds + 6 * si;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int o = ord_of(cc[k]);
                const int mn = __reduce_min_sync(grp, o);
                const int mx = __reduce_max_sync(grp, o);
                if (leader) { atomicMin(&cb[k], mn); atomicMax(&cb[3 + k], mx); }
            }
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) { cmin[k] = fminf(cmin[k], cc[k]); cmax[k] = fmaxf(cmax[k], cc[k]); }
        }
    }
    if (nseg > 1) return;
    // warp then block reduction of the centroid bounds
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            cmin[k] = fminf(cmin[k], __shfl_xor_sync(0xffffffffu, cmin[k], o));
            cmax[k] = fmaxf(cmax[k], __shfl_xor_sync(0xffffffffu, cmax[k], o));
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) { s_min[k][warp] = ord_of(cmin[k]); s_max[k][warp] = ord_of(cmax[k]); }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        int mn = s_min[k][0], mx = s_max[k][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { mn = min(mn, s_min[k][w]); mx = max(mx, s_max[k][w]); }
        atomicMin(&cbounds[k], mn);
        atomicMax(&cbounds[3 + k], mx);
    }
}

__device__ __forceinline__ uint64_t expand21(uint32_t v)
{
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// Morton code of each box centre over its segment's centroid bounds, with
// the segment id above it: key = seg << (3 * mbits) | morton (mbits bits per
// axis; 21 for a single scene).  The sort breaks equal keys by index.
__global__ void k_morton(const float4 *__restrict__ blo, const float4 *__restrict__ bhi, int32_t n,
                         const int32_t *__restrict__ seg, int32_t nseg, int mbits, const int *__restrict__ cbounds,
                         uint64_t *__restrict__ keys, int32_t *__restrict__ vals)
{
    const float qmax = (float)((1u << mbits) - 1u);
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t s = (nseg > 1) ? seg[i] : 0;
        const int *cb = cbounds + 6 * s;
        const float4 a = blo[i], b = bhi[i];
        const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
        uint32_t q[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float lo = of_ord(cb[k]);
            const float ext = of_ord(cb[3 + k]) - lo;
            const float sc = (ext > 0.f) ? qmax / ext : 0.f;
            q[k] = (uint32_t)fminf(fmaxf((c[k] - lo) * sc, 0.f), qmax);
        }
        const uint64_t m = expand21(q[0]) | (expand21(q[1]) << 1) | (expand21(q[2]) << 2);
        keys[i] = ((uint64_t)s << (3 * mbits)) | m;
        vals[i] = i;
    }
}

// Common-prefix length of sorted keys i and j, index-extended for equal keys.
__device__ __forceinline__ int delta(const uint64_t *__restrict__ keys, int32_t n, int32_t i, int32_t j)
{
    if (j < 0 || j >= n) return -1;
    const uint64_t a = keys[i], b = keys[j];
    if (a != b) return __clzll((long long)(a ^ b));
    return 64 + __clz((int)((uint32_t)i ^ (uint32_t)j));
}

// Binary radix tree over the sorted keys (Karras 2012, section 4).
// Child refs: >= 0 internal node, < 0 leaf ~k (sorted position k).
__global__ void k_karras(const uint64_t *__restrict__ keys, int32_t n, int32_t *__restrict__ left,
                         int32_t *__restrict__ right, int32_t *__restrict__ first, int32_t *__restrict__ last,
                         int32_t *__restrict__ count, int32_t *__restrict__ parent, int32_t *__restrict__ leaf_parent)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int32_t lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int32_t l = 0;
    for (int32_t t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int32_t j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int32_t s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int32_t gamma = i + s * d + min(d, 0);
    const int32_t lo = min(i, j), hi = max(i, j);
    const int32_t lref = (lo == gamma) ? ~gamma : gamma;
    const int32_t rref = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    left[i] = lref;
    right[i] = rref;
    first[i] = lo;
    last[i] = hi;
    count[i] = hi - lo + 1;
    if (lref < 0) leaf_parent[~lref] = i; else parent[lref] = i;
    if (rref < 0) leaf_parent[~rref] = i; else parent[rref] = i;
    if (i == 0) parent[0] = -1;
}

// Leaf boxes in sorted order.
__global__ void k_leaf_boxes(const int32_t *__restrict__ vals, int32_t n, const float4 *__restrict__ blo,
                             const float4 *__restrict__ bhi, float4 *__restrict__ llo, float4 *__restrict__ lhi)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int32_t t = vals[k];
    llo[k] = blo[t];
    lhi[k] = bhi[t];
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi)
{
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dx * dz + dy * dz;
}

// ------------------------------------------------- surface-area collapse
//
// Cost model of the 8-wide tree (Ylitie, Karras & Laine, HPG 2017, section
// 3): visiting a wide node costs its surface area times kCostNode, a leaf
// slot its area times kCostTri per triangle.  For every binary node n and
// i = 1..8, C(n, i) is the least cost of representing n's subtree with at
// most i slots of the parent: C(n, 1) = min(leaf, wide node = area * kCostNode
// + D(n, 8)), C(n, i) = min(C(n, i - 1), D(n, i)), where D(n, j) = min over
// k of C(left, k) + C(right, j - k).  The tables are built bottom-up with the
// tree; the collapse then distributes each wide node's 8 slots by them.
// Decision word of a node: bits 3(i-2)..3(i-2)+2 the left share k of D(n, i)
// when C(n, i) takes it (0: C(n, i) = C(n, i - 1)), bits 21..23 the left share
// of D(n, 8), bit 31 set when one slot holds n as a leaf.
#ifndef RT_COLLAPSE_SAH
#define RT_COLLAPSE_SAH 1
#endif
#ifndef RT_SAH_COST_TRI
#define RT_SAH_COST_TRI 0.6f
#endif
constexpr float kCostNode = 1.0f;
constexpr float kCostTri = RT_SAH_COST_TRI;

// Cost table of a child ref (a leaf triangle or an internal node).
__device__ __forceinline__ void sah_child(const float *sah, int32_t ref, float4 lo, float4 hi, float *c)
{
    if (ref < 0) {
        const float v = half_area(lo, hi) * kCostTri;
#pragma unroll
        for (int i = 0; i < 8; ++i) c[i] = v;
        return;
    }
    const float4 *p = reinterpret_cast<const float4 *>(sah + 8 * (size_t)ref);
    const float4 x = __ldcg(p), y = __ldcg(p + 1);
    c[0] = x.x; c[1] = x.y; c[2] = x.z; c[3] = x.w;
    c[4] = y.x; c[5] = y.y; c[6] = y.z; c[7] = y.w;
}

// Table and decision word of internal node id from its children's tables.
__device__ __forceinline__ void sah_node(float *sah, uint32_t *dec, int32_t id, float area, int32_t count,
                                         const float *cl, const float *cr, float *row = nullptr)
{
    float dist[9];
    uint32_t split[9];
#pragma unroll
    for (int j = 2; j <= 8; ++j) {
        float best = __int_as_float(0x7f800000);
        uint32_t bk = 1;
#pragma unroll
        for (int k = 1; k < j; ++k) {
            const float v = cl[k - 1] + cr[j - k - 1];
            if (v < best) { best = v; bk = (uint32_t)k; }
        }
        dist[j] = best;
        split[j] = bk;
    }
    const float cint = dist[8] + area * kCostNode;
    const float cleaf = count <= kMaxLeafTris ? area * kCostTri * (float)count : __int_as_float(0x7f800000);
    float c[8];
    uint32_t d = split[8] << 21;
    c[0] = fminf(cleaf, cint);
    if (cleaf <= cint) d |= 1u << 31;
#pragma unroll
    for (int i = 2; i <= 8; ++i) {
        if (dist[i] < c[i - 2]) {
            c[i - 1] = dist[i];
            d |= split[i] << (3 * (i - 2));
        } else {
            c[i - 1] = c[i - 2];
        }
    }
    float4 *p = reinterpret_cast<float4 *>(sah + 8 * (size_t)id);
    __stcg(p, make_float4(c[0], c[1], c[2], c[3]));
    __stcg(p + 1, make_float4(c[4], c[5], c[6], c[7]));
    __stcg(dec + id, d);
    if (row) {
#pragma unroll
        for (int i = 0; i < 8; ++i) row[i] = c[i];
    }
}

// atomicAdd with acquire-release order at device scope: the caller's
// earlier stores are visible to whoever later reads the counter, and the
// caller sees everything released before the value it reads.
__device__ __forceinline__ int atomic_add_acq_rel(int32_t *p, int32_t v)
{
    int32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

constexpr int kRefitMaxDepth = 1 << 16;   // binary levels a refit walk may climb
constexpr int32_t kEmptySlot = INT32_MIN;

// Bottom-up box refit from one child up: the second child to arrive at a
// node unions both and goes on.  The climbing child's ref, box and
// surface-area row stay in registers; only the sibling's are loaded.
__device__ __forceinline__ void refit_climb(int32_t cur, float4 mlo, float4 mhi, float *mrow, int32_t p,
                                            const int32_t *__restrict__ left, const int32_t *__restrict__ right,
                                            const int32_t *__restrict__ parent, const float4 *__restrict__ llo,
                                            const float4 *__restrict__ lhi, float4 *ilo, float4 *ihi,
                                            int32_t *flags, const int32_t *__restrict__ count, float *sah,
                                            uint32_t *dec, int32_t *err)
{
    int guard = 0;
    while (p >= 0) {
        if (++guard > kRefitMaxDepth) { atomicExch(err, 1); return; }
        // releases this thread's stores for the sibling's thread; the second
        // to arrive acquires the first's
        if (atomic_add_acq_rel(&flags[p], 1) == 0) return;   // first arrival: sibling not ready
        const int32_t l = left[p], r = right[p];
        const bool from_left = l == cur;
        const int32_t sib = from_left ? r : l;
        const float4 s0 = (sib < 0) ? llo[~sib] : __ldcg(&ilo[sib]);
        const float4 s1 = (sib < 0) ? lhi[~sib] : __ldcg(&ihi[sib]);
        const float4 plo = make_float4(fminf(mlo.x, s0.x), fminf(mlo.y, s0.y), fminf(mlo.z, s0.z), 0.f);
        const float4 phi = make_float4(fmaxf(mhi.x, s1.x), fmaxf(mhi.y, s1.y), fmaxf(mhi.z, s1.z), 0.f);
        __stcg(&ilo[p], plo);
        __stcg(&ihi[p], phi);
        if (sah) {
            float srow[8], prow[8];
            sah_child(sah, sib, s0, s1, srow);
            if (from_left) sah_node(sah, dec, p, half_area(plo, phi), count[p], mrow, srow, prow);
            else sah_node(sah, dec, p, half_area(plo, phi), count[p], srow, mrow, prow);
#pragma unroll
            for (int i = 0; i < 8; ++i) mrow[i] = prow[i];
        }
        cur = p;
        mlo = plo;
        mhi = phi;
        p = parent[p];
    }
}

__global__ void k_refit(int32_t n, const int32_t *__restrict__ left, const int32_t *__restrict__ right,
                        const int32_t *__restrict__ parent, const int32_t *__restrict__ leaf_parent,
                        const float4 *__restrict__ llo, const float4 *__restrict__ lhi, float4 *ilo, float4 *ihi,
                        int32_t *flags, const int32_t *__restrict__ count, float *sah, uint32_t *dec,
                        int32_t *err)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 mlo = llo[k], mhi = lhi[k];
    float mrow[8];
    if (sah) sah_child(sah, ~k, mlo, mhi, mrow);
    refit_climb(~k, mlo, mhi, mrow, leaf_parent[k], left, right, parent, llo, lhi, ilo, ihi, flags, count, sah, dec,
                err);
}

// Root of each segment: the binary node whose range is exactly the
// segment's sorted range (the lowest common ancestor of its first and last
// leaves; keys of one segment share the segment-id prefix).  Emits one
// collapse task per non-empty segment and an empty wide node per empty one.
__global__ void k_roots(int32_t nseg, int32_t n, const int32_t *__restrict__ seg_first,
                        const int32_t *__restrict__ first, const int32_t *__restrict__ last,
                        const int32_t *__restrict__ parent, const int32_t *__restrict__ leaf_parent,
                        int2 *__restrict__ tasks, int32_t *level_count, int32_t *counters,
                        WideNode *__restrict__ nodes)
{
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const int32_t f = seg_first[s], l = seg_first[s + 1] - 1;
    if (l < f) {
        WideNode W;
        memset(&W, 0, sizeof(W));
        for (int k = 0; k < 8; ++k) { W.qlo_x[k] = W.qlo_y[k] = W.qlo_z[k] = 255; }
        nodes[s] = W;
        return;
    }
    int32_t root = ~f;
    if (nseg == 1 && l > f) {
        root = 0;   // the radix tree of one scene: node 0 spans every leaf
    } else if (l > f) {
        int32_t p = leaf_parent[f];
        int guard = 0;
        while (p >= 0 && !(first[p] <= f && last[p] >= l) && guard++ < 128) p = parent[p];
        if (p < 0 || first[p] != f || last[p] != l) { atomicExch(&counters[3], 1); return; }
        root = p;
    }
    const int slot = atomicAdd(&level_count[0], 1);
    tasks[slot] = make_int2(root, s);
    (void)n;
}


// ------------------------------------------------------------------ PLOC
//
// Clusters live in Morton order as two float4 per cluster: (lo.xyz, segment)
// and (hi.xyz, binary ref), ref >= 0 an internal node, < 0 leaf ~k (sorted
// position k).  One iteration: every cluster finds its nearest neighbour
// (smallest merged surface area, lowest index on ties) among the kPlocRadius
// clusters on either side within its segment; mutual pairs merge into a new
// internal node at the lower position; a stable compaction keeps the order.
// An iteration that merged fewer than 1/16 of the clusters makes the next
// one pair neighbours outright (alternating parity), which bounds the number
// of iterations on degenerate input (many equal distances).
//
// state: [0,1] cluster count, [2,3] next internal node id, [4,5] forced
// pairing (ping-pong by iteration parity), [6] clusters to end with (one per
// non-empty segment).
constexpr int kCollapseGroup = 12;         // collapse levels between read-backs
constexpr int kPlocRadius = 24;
constexpr int kPlocGroup = 8;              // iterations between count read-backs
constexpr int kPlocMaxIterations = 1024;
constexpr int kPlocTile = 256;
constexpr int kPlocBlock = 1024;
enum : int { kStCount = 0, kStBase = 2, kStForced = 4, kStTarget = 6, kStError = 7, kStWords = 8 };

__device__ __forceinline__ float4 box_min(float4 a, float4 b)
{
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), a.w);
}
__device__ __forceinline__ float4 box_max(float4 a, float4 b)
{
    return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), a.w);
}

// Initial clusters = the sorted leaves; segment id from the key's top bits.
__global__ void k_ploc_init(int32_t n, const uint64_t *__restrict__ keys, int seg_shift, int32_t nseg,
                            const float4 *__restrict__ llo, const float4 *__restrict__ lhi, float4 *__restrict__ cl,
                            float4 *__restrict__ ch)
{
    for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int32_t seg = (nseg > 1) ? (int32_t)(keys[k] >> seg_shift) : 0;
        const float4 a = llo[k], b = lhi[k];
        cl[k] = make_float4(a.x, a.y, a.z, __int_as_float(seg));
        ch[k] = make_float4(b.x, b.y, b.z, __int_as_float(~k));
    }
}

// Segments: empty ones get an empty wide node (every ray misses), the others
// count towards the number of clusters the iterations end with.
__global__ void k_ploc_segments(int32_t nseg, int32_t n, const int32_t *__restrict__ seg_first, int32_t *state,
                                WideNode *__restrict__ nodes)
{
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) {
        state[kStCount] = n;
        state[kStBase] = 0;
        state[kStForced] = 0;
    }
    if (s >= nseg) return;
    if (seg_first[s + 1] > seg_first[s]) {
        atomicAdd(&state[kStTarget], 1);
        return;
    }
    WideNode W;
    memset(&W, 0, sizeof(W));
    for (int k = 0; k < 8; ++k) { W.qlo_x[k] = W.qlo_y[k] = W.qlo_z[k] = 255; }
    nodes[s] = W;
}

// Nearest neighbours of a tile of kPlocTile clusters.  The merged-box
// surface area is symmetric, so each pair is evaluated once: every row of the
// tile and the kPlocRadius rows before it computes its distances to the
// kPlocRadius clusters after it (dist, rows padded to an odd stride against
// bank conflicts), and each cluster then scans its backward distances (from
// the rows before it) and its forward ones in increasing neighbour order,
// keeping the first smallest, exactly as a full two-sided scan would.
constexpr int kPlocRow = kPlocRadius + 1;

__global__ void __launch_bounds__(kPlocTile) k_ploc_nn(const float4 *__restrict__ cl, const float4 *__restrict__ ch,
                                                      int32_t *__restrict__ nn, const int32_t *__restrict__ state,
                                                      int it)
{
    __shared__ float4 slo[kPlocTile + 2 * kPlocRadius], shi[kPlocTile + 2 * kPlocRadius];
    __shared__ float dist[(kPlocTile + kPlocRadius) * kPlocRow];
    const int par = it & 1;
    const int32_t count = state[kStCount + par];
    const int32_t b0 = blockIdx.x * kPlocTile;
    if (b0 >= count) return;
    const bool done = count <= state[kStTarget];
    const bool forced = state[kStForced + par] != 0;
    for (int k = threadIdx.x; k < kPlocTile + 2 * kPlocRadius; k += kPlocTile) {
        const int32_t g = b0 - kPlocRadius + k;
        if (g >= 0 && g < count) {
            slo[k] = cl[g];
            shi[k] = ch[g];
        }
    }
    __syncthreads();
    const float inf = __int_as_float(0x7f800000);
    if (!done && !forced) {
        // forward distances of rows r = 0 .. kPlocTile + kPlocRadius - 1
        // (cluster b0 - kPlocRadius + r) to the kPlocRadius clusters after it
        for (int r = threadIdx.x; r < kPlocTile + kPlocRadius; r += kPlocTile) {
            const int32_t g = b0 - kPlocRadius + r;
            float *row = dist + r * kPlocRow;
            if (g < 0 || g >= count) {
                for (int k = 0; k < kPlocRadius; ++k) row[k] = inf;
                continue;
            }
            const float4 a0 = slo[r], a1 = shi[r];
            const int seg = __float_as_int(a0.w);
#pragma unroll 4
            for (int k = 1; k <= kPlocRadius; ++k) {
                float d = inf;
                if (g + k < count) {
                    const float4 b0v = slo[r + k];
                    if (__float_as_int(b0v.w) == seg) d = half_area(box_min(a0, b0v), box_max(a1, shi[r + k]));
                }
                row[k - 1] = d;
            }
        }
    }
    __syncthreads();
    const int32_t i = b0 + threadIdx.x;
    if (i >= count) return;
    int32_t best = -1;
    if (!done) {
        const int t = threadIdx.x + kPlocRadius;
        if (forced) {
            const int seg = __float_as_int(slo[t].w);
            const int32_t p = ((i - par) ^ 1) + par;
            if (i - par >= 0 && p >= 0 && p < count && __float_as_int(slo[t + (p - i)].w) == seg) best = p;
        } else {
            float bd = inf;
            for (int k = kPlocRadius; k >= 1; --k) {   // neighbours i - k, nearest last
                const float d = dist[(t - k) * kPlocRow + (k - 1)];
                if (d < bd) { bd = d; best = i - k; }
            }
            for (int k = 1; k <= kPlocRadius; ++k) {   // neighbours i + k
                const float d = dist[t * kPlocRow + (k - 1)];
                if (d < bd) { bd = d; best = i + k; }
            }
        }
    }
    nn[i] = best;
}

// 0/1 flags of cluster i: survives (not absorbed by a lower partner) and
// creates a node (lower half of a mutual pair).
__device__ __forceinline__ void ploc_flags(const int32_t *__restrict__ nn, int32_t i, int32_t count, bool &keep,
                                           bool &make)
{
    keep = false;
    make = false;
    if (i >= count) return;
    const int32_t j = nn[i];
    const bool mutual = j >= 0 && nn[j] == i;
    keep = !(mutual && i > j);
    make = mutual && i < j;
}

// Exclusive block prefix of two 0/1 flags (1024 threads); totals in *tk, *tm.
__device__ __forceinline__ void block_prefix2(bool keep, bool make, int &pk, int &pm, int &tk, int &tm)
{
    __shared__ int wk[32], wm[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t bk = __ballot_sync(0xffffffffu, keep), bm = __ballot_sync(0xffffffffu, make);
    const uint32_t below = (1u << lane) - 1u;
    if (lane == 0) { wk[warp] = __popc(bk); wm[warp] = __popc(bm); }
    __syncthreads();
    if (warp == 0) {
        int vk = wk[lane], vm = wm[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int uk = __shfl_up_sync(0xffffffffu, vk, o), um = __shfl_up_sync(0xffffffffu, vm, o);
            if (lane >= o) { vk += uk; vm += um; }
        }
        wk[lane] = vk;
        wm[lane] = vm;
    }
    __syncthreads();
    pk = (warp ? wk[warp - 1] : 0) + __popc(bk & below);
    pm = (warp ? wm[warp - 1] : 0) + __popc(bm & below);
    tk = wk[31];
    tm = wm[31];
}

__global__ void __launch_bounds__(kPlocBlock) k_ploc_count(const int32_t *__restrict__ nn,
                                                          const int32_t *__restrict__ state, int it,
                                                          int2 *__restrict__ bsum)
{
    const int32_t count = state[kStCount + (it & 1)];
    if ((int32_t)blockIdx.x * kPlocBlock >= count) return;
    const int32_t i = blockIdx.x * kPlocBlock + threadIdx.x;
    bool keep, make;
    ploc_flags(nn, i, count, keep, make);
    int pk, pm, tk, tm;
    block_prefix2(keep, make, pk, pm, tk, tm);
    if (threadIdx.x == 0) bsum[blockIdx.x] = make_int2(tk, tm);
}

// One block: exclusive scan of the per-block totals, next count / node base
// / pairing mode.
__global__ void __launch_bounds__(kPlocBlock) k_ploc_scan(int2 *__restrict__ bsum, int32_t *state, int it)
{
    const int par = it & 1;
    const int32_t count = state[kStCount + par];
    const int32_t nb = (count + kPlocBlock - 1) / kPlocBlock;
    const int32_t per = (nb + kPlocBlock - 1) / kPlocBlock;
    const int32_t lo = threadIdx.x * per, hi = min(lo + per, nb);
    int sk = 0, sm = 0;
    for (int32_t b = lo; b < hi; ++b) { sk += bsum[b].x; sm += bsum[b].y; }
    __shared__ int xk[kPlocBlock], xm[kPlocBlock];
    xk[threadIdx.x] = sk;
    xm[threadIdx.x] = sm;
    __syncthreads();
    for (int o = 1; o < kPlocBlock; o <<= 1) {
        const int ak = threadIdx.x >= o ? xk[threadIdx.x - o] : 0;
        const int am = threadIdx.x >= o ? xm[threadIdx.x - o] : 0;
        __syncthreads();
        xk[threadIdx.x] += ak;
        xm[threadIdx.x] += am;
        __syncthreads();
    }
    int rk = xk[threadIdx.x] - sk, rm = xm[threadIdx.x] - sm;
    for (int32_t b = lo; b < hi; ++b) {
        const int2 v = bsum[b];
        bsum[b] = make_int2(rk, rm);
        rk += v.x;
        rm += v.y;
    }
    if (threadIdx.x == kPlocBlock - 1) {
        const int total_k = xk[kPlocBlock - 1], total_m = xm[kPlocBlock - 1];
        state[kStCount + (par ^ 1)] = total_k;
        state[kStBase + (par ^ 1)] = state[kStBase + par] + total_m;
        state[kStForced + (par ^ 1)] = (count > state[kStTarget] && total_m * 16 < count) ? 1 : 0;
    }
}

__global__ void __launch_bounds__(kPlocBlock) k_ploc_merge(const float4 *__restrict__ cl, const float4 *__restrict__ ch,
                                                          float4 *__restrict__ cl2, float4 *__restrict__ ch2,
                                                          const int32_t *__restrict__ nn,
                                                          const int2 *__restrict__ boff,
                                                          const int32_t *__restrict__ state, int it,
                                                          int32_t *__restrict__ left, int32_t *__restrict__ right,
                                                          int32_t *__restrict__ ncount, float4 *__restrict__ ilo,
                                                          float4 *__restrict__ ihi, float *sah, uint32_t *dec,
                                                          int32_t *__restrict__ parent,
                                                          int32_t *__restrict__ leaf_parent)
{
    const int par = it & 1;
    const int32_t count = state[kStCount + par];
    if ((int32_t)blockIdx.x * kPlocBlock >= count) return;
    const int32_t i = blockIdx.x * kPlocBlock + threadIdx.x;
    bool keep, make;
    ploc_flags(nn, i, count, keep, make);
    int pk, pm, tk, tm;
    block_prefix2(keep, make, pk, pm, tk, tm);
    if (!keep) return;
    const int2 bo = boff[blockIdx.x];
    const int32_t pos = bo.x + pk;
    float4 a0 = cl[i], a1 = ch[i];
    if (make) {
        const int32_t j = nn[i];
        const float4 b0 = cl[j], b1 = ch[j];
        const int32_t id = state[kStBase + par] + bo.y + pm;
        const int32_t l = __float_as_int(a1.w), r = __float_as_int(b1.w);
        left[id] = l;
        right[id] = r;
        if (l < 0) leaf_parent[~l] = id; else parent[l] = id;
        if (r < 0) leaf_parent[~r] = id; else parent[r] = id;
        const int32_t cnt = (l < 0 ? 1 : ncount[l]) + (r < 0 ? 1 : ncount[r]);
        ncount[id] = cnt;
        float cl[8], cr[8];
        if (sah) {
            sah_child(sah, l, a0, a1, cl);
            sah_child(sah, r, b0, b1, cr);
        }
        a0 = box_min(a0, b0);
        a1 = box_max(a1, b1);
        if (sah) sah_node(sah, dec, id, half_area(a0, a1), cnt, cl, cr);
        ilo[id] = make_float4(a0.x, a0.y, a0.z, 0.f);
        ihi[id] = make_float4(a1.x, a1.y, a1.z, 0.f);
        a1.w = __int_as_float(id);
    }
    cl2[pos] = a0;
    ch2[pos] = a1;
}

// The last iterations, once at most kPlocTailMax clusters remain: one
// block holds every cluster in shared memory and runs the same iteration
// (nearest neighbour, mutual pairs, stable compaction, forced pairing after
// a slow iteration) with block barriers instead of kernel boundaries.  The
// final clusters go back to (cl, ch) and the count to the state slot of
// iteration `it`'s parity.
constexpr int kPlocTailMax = 4096;
constexpr int kPlocTailItems = kPlocTailMax / kPlocBlock;
constexpr int kPlocTailMaxIterations = 4096;

__global__ void __launch_bounds__(kPlocBlock) k_ploc_tail(float4 *__restrict__ cl, float4 *__restrict__ ch,
                                                         int32_t *state, int it, int32_t *__restrict__ left,
                                                         int32_t *__restrict__ right, int32_t *__restrict__ ncount,
                                                         float4 *__restrict__ ilo, float4 *__restrict__ ihi,
                                                         float *sah, uint32_t *dec, int32_t *__restrict__ parent,
                                                         int32_t *__restrict__ leaf_parent)
{
    extern __shared__ float4 tail_smem[];
    float4 *slo = tail_smem;                       // kPlocTailMax
    float4 *shi = tail_smem + kPlocTailMax;        // kPlocTailMax
    int32_t *snn = reinterpret_cast<int32_t *>(tail_smem + 2 * kPlocTailMax);   // kPlocTailMax
    __shared__ int wsum[2][32];
    __shared__ int s_count, s_base, s_forced, s_error;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int par = it & 1;
    const int32_t target = state[kStTarget];
    if (tid == 0) {
        s_count = state[kStCount + par];
        s_base = state[kStBase + par];
        s_forced = state[kStForced + par];
        s_error = 0;
    }
    __syncthreads();
    const int32_t count0 = s_count;
    for (int k = 0; k < kPlocTailItems; ++k) {
        const int i = tid + k * kPlocBlock;
        if (i < count0) { slo[i] = cl[i]; shi[i] = ch[i]; }
    }
    __syncthreads();
    for (int step = 0; step < kPlocTailMaxIterations; ++step) {
        const int32_t count = s_count;
        if (count <= target) break;
        const bool forced = s_forced != 0;
        const int ppar = step & 1;
        // nearest neighbours
        for (int k = 0; k < kPlocTailItems; ++k) {
            const int i = tid + k * kPlocBlock;
            if (i >= count) break;
            const float4 a0 = slo[i], a1 = shi[i];
            const int seg = __float_as_int(a0.w);
            int best = -1;
            if (forced) {
                const int p = ((i - ppar) ^ 1) + ppar;
                if (i - ppar >= 0 && p >= 0 && p < count && __float_as_int(slo[p].w) == seg) best = p;
            } else {
                float bd = __int_as_float(0x7f800000);
                const int j0 = max(0, i - kPlocRadius), j1 = min(count - 1, i + kPlocRadius);
                for (int j = j0; j <= j1; ++j) {
                    if (j == i) continue;
                    const float4 b0 = slo[j];
                    if (__float_as_int(b0.w) != seg) continue;
                    const float d = half_area(box_min(a0, b0), box_max(a1, shi[j]));
                    if (d < bd) { bd = d; best = j; }
                }
            }
            snn[i] = best;
        }
        __syncthreads();
        // flags, per-thread totals, block scan
        bool keep[kPlocTailItems], make[kPlocTailItems];
        int tk = 0, tm = 0;
        for (int k = 0; k < kPlocTailItems; ++k) {
            const int i = tid * kPlocTailItems + k;   // contiguous items per thread keep the order
            keep[k] = make[k] = false;
            if (i < count) {
                const int j = snn[i];
                const bool mutual = j >= 0 && snn[j] == i;
                keep[k] = !(mutual && i > j);
                make[k] = mutual && i < j;
            }
            tk += keep[k];
            tm += make[k];
        }
        int ik = tk, im = tm;
        for (int o = 1; o < 32; o <<= 1) {
            const int uk = __shfl_up_sync(0xffffffffu, ik, o), um = __shfl_up_sync(0xffffffffu, im, o);
            if (lane >= o) { ik += uk; im += um; }
        }
        if (lane == 31) { wsum[0][warp] = ik; wsum[1][warp] = im; }
        __syncthreads();
        if (warp == 0) {
            int vk = wsum[0][lane], vm = wsum[1][lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int uk = __shfl_up_sync(0xffffffffu, vk, o), um = __shfl_up_sync(0xffffffffu, vm, o);
                if (lane >= o) { vk += uk; vm += um; }
            }
            wsum[0][lane] = vk;
            wsum[1][lane] = vm;
        }
        __syncthreads();
        int pk = (warp ? wsum[0][warp - 1] : 0) + ik - tk;
        int pm = (warp ? wsum[1][warp - 1] : 0) + im - tm;
        const int total_k = wsum[0][31], total_m = wsum[1][31];
        // read every surviving cluster (and its partner) before any write
        float4 v0[kPlocTailItems], v1[kPlocTailItems];
        int vpos[kPlocTailItems];
        for (int k = 0; k < kPlocTailItems; ++k) {
            const int i = tid * kPlocTailItems + k;
            vpos[k] = -1;
            if (!keep[k]) continue;
            float4 a0 = slo[i], a1 = shi[i];
            if (make[k]) {
                const int j = snn[i];
                const float4 b0 = slo[j], b1 = shi[j];
                const int32_t id = s_base + pm;
                ++pm;
                const int32_t l = __float_as_int(a1.w), r = __float_as_int(b1.w);
                left[id] = l;
                right[id] = r;
                if (l < 0) leaf_parent[~l] = id; else parent[l] = id;
                if (r < 0) leaf_parent[~r] = id; else parent[r] = id;
                const int32_t cnt = (l < 0 ? 1 : ncount[l]) + (r < 0 ? 1 : ncount[r]);
                ncount[id] = cnt;
                float cla[8], cra[8];
                if (sah) {
                    sah_child(sah, l, a0, a1, cla);
                    sah_child(sah, r, b0, b1, cra);
                }
                a0 = box_min(a0, b0);
                a1 = box_max(a1, b1);
                if (sah) sah_node(sah, dec, id, half_area(a0, a1), cnt, cla, cra);
                ilo[id] = make_float4(a0.x, a0.y, a0.z, 0.f);
                ihi[id] = make_float4(a1.x, a1.y, a1.z, 0.f);
                a1.w = __int_as_float(id);
            }
            v0[k] = a0;
            v1[k] = a1;
            vpos[k] = pk++;
        }
        __syncthreads();
        for (int k = 0; k < kPlocTailItems; ++k)
            if (vpos[k] >= 0) { slo[vpos[k]] = v0[k]; shi[vpos[k]] = v1[k]; }
        if (tid == 0) {
            s_count = total_k;
            s_base += total_m;
            s_forced = (total_m * 16 < count) ? 1 : 0;
            if (step == kPlocTailMaxIterations - 1 && total_k > target) s_error = 1;
        }
        __syncthreads();
    }
    const int32_t count = s_count;
    for (int k = 0; k < kPlocTailItems; ++k) {
        const int i = tid + k * kPlocBlock;
        if (i < count) { cl[i] = slo[i]; ch[i] = shi[i]; }
    }
    if (tid == 0) {
        state[kStCount + par] = count;
        state[kStBase + par] = s_base;
        if (s_error) state[kStError] = 1;
    }
}

// ---------------------------------------------------------------- H-PLOC
//
// Hierarchical PLOC (Benthin, Meister, Barczak, Mohan, Oldfield, HPG 2024):
// the clustering of PLOC without global iterations.  Every leaf climbs the
// Morton radix tree bottom-up (Apetrei 2014: the parent of the node covering
// sorted positions [L, R] sits at whichever boundary split, L - 1 or R, has
// the longer common key prefix; the second of the two children to arrive
// goes on, the first stops).  A subtree of at most kHplocKeep leaves is its
// leaves (nothing merged, nothing stored); a larger one is at most
// kHplocKeep clusters, stored as binary refs (>= 0 internal node, < 0 leaf
// ~k) at the start of its range in `cref`.  At a parent of more than
// kHplocKeep leaves (or the root) the warp loads the two children's refs and
// boxes one per lane and, while more than kHplocKeep remain (one at the
// root), merges every mutual nearest-neighbour pair among the RT_HPLOC_RADIUS
// clusters on either side in Morton order (smallest merged surface area,
// lowest index on ties -- the smallest such pair is always mutual); then it
// stores the refs at the start of the parent's range.  Warps serve their
// lanes' parents one after another with all 32 lanes; the node ids of a
// parent's merges are reserved with one atomic (one more when the last
// round merges past kHplocKeep).  The stores a level leaves for the parents above are fenced before
// the next 64-bit exchange that tells a parent which child came first, and
// read after a fence that follows it (through L2).  Single-scene builds;
// nodes, counts and surface-area tables as the PLOC kernels write them
// (an internal node's box also carries its triangle count in .w).
#ifndef RT_HPLOC_KEEP
#define RT_HPLOC_KEEP 16
#endif
constexpr int kHplocKeep = RT_HPLOC_KEEP;
static_assert(2 * kHplocKeep <= 32, "the two children's clusters must fit one warp");
// One warp per block, 64 registers: a block's resources free as soon as its
// warp's lanes have all stopped climbing (measured: 4 % faster than 64- and
// 128-thread blocks, 30 % faster than 256 threads at 75 registers).
#ifndef RT_HPLOC_BLOCK
#define RT_HPLOC_BLOCK 32
#endif
#ifndef RT_HPLOC_MIN_BLOCKS
#define RT_HPLOC_MIN_BLOCKS 32
#endif
constexpr int kHplocBlock = RT_HPLOC_BLOCK;
// neighbours searched on either side in Morton order (>= 31: all of them);
// 3 measured best: 2 builds 2 % faster but renders the terrain 5 % slower,
// 4..6 build 3..10 % slower and render no faster (all: 1.3x the build time)
#ifndef RT_HPLOC_RADIUS
#define RT_HPLOC_RADIUS 3
#endif
constexpr unsigned long long kHplocEmpty = ~0ull;
// Carry each cluster's surface-area cost row in registers through the merges
// (shuffled with its box) instead of loading the children's rows from the
// table at every merge.
#ifndef RT_HPLOC_ROWS
#define RT_HPLOC_ROWS 1
#endif

// Is the pair (a, a + 1) of sorted keys closer (longer common prefix) than
// (b, b + 1)?  Equal keys fall back to the positions' xor (balanced trees
// over runs of equal codes), then to the positions themselves: a strict
// total order, so every split has exactly two children.
__device__ __forceinline__ bool hploc_closer(const uint64_t *__restrict__ keys, int32_t a, int32_t b)
{
    const uint64_t ka = __ldg(keys + a) ^ __ldg(keys + a + 1), kb = __ldg(keys + b) ^ __ldg(keys + b + 1);
    if (ka != kb) return ka < kb;
    const uint32_t ia = (uint32_t)a ^ (uint32_t)(a + 1), ib = (uint32_t)b ^ (uint32_t)(b + 1);
    if (ia != ib) return ia < ib;
    return a < b;
}

__global__ void k_hploc_init(int32_t n, unsigned long long *__restrict__ meet)
{
    for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        meet[k] = kHplocEmpty;
}

__global__ void __launch_bounds__(kHplocBlock, RT_HPLOC_MIN_BLOCKS) k_hploc(int32_t n, const uint64_t *__restrict__ keys,
                                                       int32_t *__restrict__ cref,
                                                       unsigned long long *__restrict__ meet, int32_t *state,
                                                       const float4 *__restrict__ llo, const float4 *__restrict__ lhi,
                                                       float4 *__restrict__ cl, float4 *__restrict__ ch,
                                                       int32_t *__restrict__ left, int32_t *__restrict__ right,
                                                       int32_t *__restrict__ ncount, float4 *__restrict__ ilo,
                                                       float4 *__restrict__ ihi, float *sah, uint32_t *dec,
                                                       int32_t *__restrict__ parent,
                                                       int32_t *__restrict__ leaf_parent)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t below = (1u << lane) - 1u;
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t ninternal = n - 1;
    int32_t L = i, R = i, nc = 1;          // the lane's subtree: range and cluster count
    bool active = i < n && n > 1;
    bool bad = false;
    int guard = 0;
    while (__any_sync(0xffffffffu, active)) {
        // climb one level: the parent split and who arrived first
        bool go_on = false, root = false;
        int32_t lpos = 0, nl = 0, rpos = 0, nr = 0;
        if (active) {
            const bool go_right = (L == 0) || (R != n - 1 && hploc_closer(keys, R, L - 1));
            const int32_t split = go_right ? R : L - 1;
            const unsigned long long mine =
                ((unsigned long long)(uint32_t)(go_right ? L : R) << 32) | (uint32_t)nc;
            const unsigned long long other = atomicExch(&meet[split], mine);
            if (other == kHplocEmpty) {
                active = false;                  // the sibling's lane goes on
            } else {
                const int32_t far = (int32_t)(other >> 32), sn = (int32_t)(uint32_t)other;
                if (go_right) {                  // this lane holds the left child [L, split]
                    lpos = L; nl = nc; rpos = split + 1; nr = sn;
                    R = far;
                } else {                         // the left child is [far, split]
                    lpos = far; nl = sn; rpos = L; nr = nc;
                    L = far;
                }
                if (L < 0 || R >= n || L > R || nl < 1 || nr < 1 || nl > kHplocKeep || nr > kHplocKeep ||
                    nl > rpos - lpos || nr > R - rpos + 1) {
                    bad = true;                  // never expected; keeps every access in bounds
                    active = false;
                } else {
                    root = (L == 0 && R == n - 1);
                    if (root || R - L + 1 > kHplocKeep) {
                        __threadfence();         // the children's stored refs and nodes
                        go_on = true;
                    } else {
                        nc = nl + nr;            // still its leaves
                    }
                }
            }
        }
        __syncwarp();
        // the warp serves each of its lanes' parents in turn
        uint32_t todo = __ballot_sync(0xffffffffu, go_on);
        const bool stored = todo != 0u;
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const int32_t p_l = __shfl_sync(0xffffffffu, lpos, src), p_nl = __shfl_sync(0xffffffffu, nl, src);
            const int32_t p_r = __shfl_sync(0xffffffffu, rpos, src), p_nr = __shfl_sync(0xffffffffu, nr, src);
            const int32_t p_end = __shfl_sync(0xffffffffu, R, src);
            const bool p_root = __shfl_sync(0xffffffffu, root, src);
            int cnt = p_nl + p_nr;
            bool valid = (int)lane < cnt;
            int32_t ref = 0;
            float4 c0 = make_float4(0.f, 0.f, 0.f, 0.f), c1 = c0;
#if RT_HPLOC_ROWS
            float row[8];                        // the cluster's surface-area cost row
#pragma unroll
            for (int q = 0; q < 8; ++q) row[q] = 0.f;
#endif
            if (valid) {
                // a child of as many leaves as clusters is its leaves; else its refs are stored
                const bool in_left = (int)lane < p_nl;
                const int32_t g = in_left ? p_l + (int32_t)lane : p_r + ((int32_t)lane - p_nl);
                const bool leaves = in_left ? p_nl == p_r - p_l : p_nr == p_end - p_r + 1;
                ref = leaves ? ~g : __ldcg(cref + g);
                if (ref >= ninternal || ref < -n) { bad = true; ref = ~0; }
                if (ref < 0) {
                    c0 = __ldg(llo + ~ref);
                    c1 = __ldg(lhi + ~ref);
                    c0.w = __int_as_float(1);
                } else {
                    c0 = __ldcg(ilo + ref);      // .w: the node's triangle count
                    c1 = __ldcg(ihi + ref);
                }
#if RT_HPLOC_ROWS
                if (sah) sah_child(sah, ref, c0, c1, row);
#endif
            }
            const int target = p_root ? 1 : kHplocKeep;
            int32_t base = 0, extra = 0, made = 0;
            const int32_t reserved = cnt > target ? cnt - target : 0;
            if (reserved > 0) {
                if (lane == 0) base = atomicAdd(&state[kStBase], reserved);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base < 0 || base > ninternal - reserved) { bad = true; cnt = 0; valid = false; }
            }
            while (cnt > target) {
                if (++guard > 65536) {           // never expected: a mutual pair always merges
                    bad = true;
                    break;
                }
                // nearest neighbour among the cnt clusters
                float best = __int_as_float(0x7f800000);
                int bk = (int)lane;
#if RT_HPLOC_RADIUS >= 31
                for (int k = 0; k < cnt; ++k) {
                    const float ox = __shfl_sync(0xffffffffu, c0.x, k), oy = __shfl_sync(0xffffffffu, c0.y, k);
                    const float oz = __shfl_sync(0xffffffffu, c0.z, k);
                    const float px = __shfl_sync(0xffffffffu, c1.x, k), py = __shfl_sync(0xffffffffu, c1.y, k);
                    const float pz = __shfl_sync(0xffffffffu, c1.z, k);
                    if (valid && k != (int)lane) {
                        const float dx = fmaxf(c1.x, px) - fminf(c0.x, ox);
                        const float dy = fmaxf(c1.y, py) - fminf(c0.y, oy);
                        const float dz = fmaxf(c1.z, pz) - fminf(c0.z, oz);
                        const float a = dx * dy + dx * dz + dy * dz;
                        if (a < best) { best = a; bk = k; }
                    }
                }
#else
                // the merged area is symmetric: each lane forms it with the
                // RT_HPLOC_RADIUS lanes above it and takes the ones below it
                // from them; candidates visited in increasing index order
                float up[RT_HPLOC_RADIUS];
#pragma unroll
                for (int d = 1; d <= RT_HPLOC_RADIUS; ++d) {
                    const int from = ((int)lane + d) & 31;
                    const float ox = __shfl_sync(0xffffffffu, c0.x, from), oy = __shfl_sync(0xffffffffu, c0.y, from);
                    const float oz = __shfl_sync(0xffffffffu, c0.z, from);
                    const float px = __shfl_sync(0xffffffffu, c1.x, from), py = __shfl_sync(0xffffffffu, c1.y, from);
                    const float pz = __shfl_sync(0xffffffffu, c1.z, from);
                    const float dx = fmaxf(c1.x, px) - fminf(c0.x, ox);
                    const float dy = fmaxf(c1.y, py) - fminf(c0.y, oy);
                    const float dz = fmaxf(c1.z, pz) - fminf(c0.z, oz);
                    up[d - 1] = dx * dy + dx * dz + dy * dz;
                }
#pragma unroll
                for (int d = RT_HPLOC_RADIUS; d >= 1; --d) {
                    const float a = __shfl_sync(0xffffffffu, up[d - 1], ((int)lane - d) & 31);
                    if (valid && (int)lane - d >= 0 && a < best) { best = a; bk = (int)lane - d; }
                }
#pragma unroll
                for (int d = 1; d <= RT_HPLOC_RADIUS; ++d)
                    if (valid && (int)lane + d < cnt && up[d - 1] < best) { best = up[d - 1]; bk = (int)lane + d; }
#endif
                const int back = __shfl_sync(0xffffffffu, bk, bk);
                const bool mutual = valid && bk != (int)lane && back == (int)lane;
                // the lower lane of a pair makes the node
                const bool make = mutual && (int)lane < bk;
                const bool drop = mutual && (int)lane > bk;
                const uint32_t mm = __ballot_sync(0xffffffffu, make);
                const int over = made + __popc(mm) - reserved;
                if (over > 0) {                  // merged past kHplocKeep: ids for the rest
                    int32_t more = 0;
                    if (lane == 0) more = atomicAdd(&state[kStBase], over);
                    more = __shfl_sync(0xffffffffu, more, 0);
                    if (more < 0 || more > ninternal - over) { bad = true; break; }
                    extra = more - reserved;     // id of merge m >= reserved: extra + m
                }
                const float4 b0 = make_float4(__shfl_sync(0xffffffffu, c0.x, bk),
                                              __shfl_sync(0xffffffffu, c0.y, bk),
                                              __shfl_sync(0xffffffffu, c0.z, bk),
                                              __shfl_sync(0xffffffffu, c0.w, bk));
                const float4 b1 = make_float4(__shfl_sync(0xffffffffu, c1.x, bk),
                                              __shfl_sync(0xffffffffu, c1.y, bk),
                                              __shfl_sync(0xffffffffu, c1.z, bk), 0.f);
                const int32_t rb = __shfl_sync(0xffffffffu, ref, bk);
#if RT_HPLOC_ROWS
                float rowb[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) rowb[q] = __shfl_sync(0xffffffffu, row[q], bk);
#endif
                if (make) {
                    const int32_t m = made + __popc(mm & below);
                    const int32_t id = m < reserved ? base + m : extra + m;
                    const int32_t l = ref, r = rb;
                    left[id] = l;
                    right[id] = r;
                    if (l < 0) leaf_parent[~l] = id; else parent[l] = id;
                    if (r < 0) leaf_parent[~r] = id; else parent[r] = id;
                    const int32_t count = __float_as_int(c0.w) + __float_as_int(b0.w);
                    __stcg(ncount + id, count);
#if RT_HPLOC_ROWS
                    c0 = box_min(c0, b0);
                    c1 = box_max(c1, b1);
                    c0.w = __int_as_float(count);
                    if (sah) {
                        float prow[8];
                        sah_node(sah, dec, id, half_area(c0, c1), count, row, rowb, prow);
#pragma unroll
                        for (int q = 0; q < 8; ++q) row[q] = prow[q];
                    }
#else
                    float sl[8], sr[8];
                    if (sah) {
                        sah_child(sah, l, c0, c1, sl);
                        sah_child(sah, r, b0, b1, sr);
                    }
                    c0 = box_min(c0, b0);
                    c1 = box_max(c1, b1);
                    c0.w = __int_as_float(count);
                    if (sah) sah_node(sah, dec, id, half_area(c0, c1), count, sl, sr);
#endif
                    __stcg(ilo + id, c0);
                    __stcg(ihi + id, make_float4(c1.x, c1.y, c1.z, 0.f));
                    ref = id;
                }
                made += __popc(mm);
                // stable compaction of the kept clusters
                const uint32_t km = __ballot_sync(0xffffffffu, valid && !drop);
                const int kc = __popc(km);
                const int from = (int)lane < kc ? (int)__fns(km, 0, (int)lane + 1) : (int)lane;
                c0 = make_float4(__shfl_sync(0xffffffffu, c0.x, from), __shfl_sync(0xffffffffu, c0.y, from),
                                 __shfl_sync(0xffffffffu, c0.z, from), __shfl_sync(0xffffffffu, c0.w, from));
                c1 = make_float4(__shfl_sync(0xffffffffu, c1.x, from), __shfl_sync(0xffffffffu, c1.y, from),
                                 __shfl_sync(0xffffffffu, c1.z, from), 0.f);
                ref = __shfl_sync(0xffffffffu, ref, from);
#if RT_HPLOC_ROWS
#pragma unroll
                for (int q = 0; q < 8; ++q) row[q] = __shfl_sync(0xffffffffu, row[q], from);
#endif
                if (kc == cnt) {                 // never expected: no mutual pair
                    bad = true;
                    break;
                }
                cnt = kc;
                valid = (int)lane < cnt;
            }
            if (p_root && lane == 0) {
                // the root cluster, where the roots pass looks for it
                cl[0] = make_float4(c0.x, c0.y, c0.z, __int_as_float(0));
                ch[0] = make_float4(c1.x, c1.y, c1.z, __int_as_float(ref));
            }
            if (valid && !p_root) __stcg(cref + p_l + (int32_t)lane, ref);
            if ((int)lane == src) {
                nc = cnt;
                if (p_root || cnt > target) active = false;
            }
        }
        // this level's stores reach the device before any lane's next exchange
        if (stored) __threadfence();
        __syncwarp();
    }
    if (bad) atomicExch(&state[kStError], 1);
    if (i == 0) state[kStCount] = 1;
}

// The remaining clusters (one per non-empty segment, in segment order) are
// the roots: level-0 collapse tasks (binary ref, wide node = segment).
__global__ void k_ploc_roots(const float4 *__restrict__ cl, const float4 *__restrict__ ch,
                             const int32_t *__restrict__ state, int it, int2 *__restrict__ tasks,
                             int32_t *level_count, int32_t *counters, int32_t *__restrict__ parent,
                             int32_t *__restrict__ leaf_parent)
{
    const int32_t count = state[kStCount + (it & 1)];
    const int32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c == 0) {
        level_count[0] = count;
        if (count != state[kStTarget]) atomicExch(&counters[3], 1);
    }
    if (c >= count) return;
    const int32_t root = __float_as_int(ch[c].w);
    if (root < 0) leaf_parent[~root] = -1; else parent[root] = -1;
    tasks[c] = make_int2(root, __float_as_int(cl[c].w));
}

// Exponent e (biased as a float exponent) of the power-of-two grid unit for
// an extent, with room for 252 units plus one unit of padding per side.
__device__ __forceinline__ int grid_exponent(float extent)
{
    const float x = __fdiv_ru(fmaxf(extent, 0.f), 252.0f);
    if (!(x > 0.f)) return 1;                       // 2^-126
    const uint32_t bits = __float_as_uint(x);
    int e = (int)((bits >> 23) & 0xffu);            // biased exponent of x
    if (e == 0) return 1;                           // subnormal -> smallest normal unit
    if (bits & 0x7fffffu) e += 1;                   // round up to a power of two
    return min(max(e, 1), 253);
}

struct BuildArgs {
    int32_t n;
    const int32_t *left, *right;
    const int32_t *count;         // leaves under each internal node
    const uint32_t *dec;          // surface-area decisions (nullptr: greedy collapse)
    int32_t *slot_ref;            // binary ref of every slot of every wide node (kEmptySlot: none)
    const float4 *ilo, *ihi, *llo, *lhi;
    const int32_t *vals;          // sorted position -> caller's triangle id
    const float *verts;
    const int3 *idx;
    const uint32_t *flags;
    WideNode *nodes;
    PackedTri *tris;
    int32_t *counters;            // [0] nodes allocated, [1] triangle slots allocated, [2] root tasks, [3] error
    const int32_t *cur_count;     // tasks of this level
    int32_t *next_count;          // tasks emitted for the next level
    const int2 *tasks_in;         // (binary ref, wide node index)
    int2 *tasks_out;
    int32_t max_nodes;
};

// Wide nodes and triangle slots allocated together: counters[0] and
// counters[1] form one 64-bit word (nodes low, slots high; both stay below
// 2^31), so a task makes one atomic instead of two on the same line.
__device__ __forceinline__ unsigned long long alloc_nodes_tris(int32_t *counters, int32_t nodes, int32_t tris)
{
    return atomicAdd(reinterpret_cast<unsigned long long *>(counters),
                     ((unsigned long long)(uint32_t)tris << 32) | (uint32_t)nodes);
}

__device__ __forceinline__ void ref_box(const BuildArgs &A, int32_t ref, float4 &lo, float4 &hi)
{
    if (ref < 0) { lo = A.llo[~ref]; hi = A.lhi[~ref]; }
    else { lo = A.ilo[ref]; hi = A.ihi[ref]; }
}
__device__ __forceinline__ int32_t ref_count(const BuildArgs &A, int32_t ref)
{
    return (ref < 0) ? 1 : A.count[ref];
}

// The (at most kMaxLeafTris) leaves under a leaf slot's binary ref, left
// first, in at most one round trip per tree level (such a subtree is at most
// two levels deep).  False when the subtree holds more leaves than that.
__device__ __forceinline__ bool leaf_refs(const BuildArgs &A, int32_t ref, int32_t *lv, int &nlv)
{
    static_assert(kMaxLeafTris == 3, "leaf_refs walks at most two levels");
    if (ref < 0) {
        lv[0] = ref;
        nlv = 1;
        return true;
    }
    const int32_t a = A.left[ref], b = A.right[ref];
    int32_t a0 = a, a1 = 0, b0 = b, b1 = 0;
    if (a >= 0) { a0 = A.left[a]; a1 = A.right[a]; }
    if (b >= 0) { b0 = A.left[b]; b1 = A.right[b]; }
    if ((a >= 0 && b >= 0) || a0 >= 0 || b0 >= 0 || (a >= 0 && a1 >= 0) || (b >= 0 && b1 >= 0)) return false;
    lv[0] = a0;
    lv[1] = a >= 0 ? a1 : b0;
    lv[2] = a >= 0 ? b0 : b1;
    nlv = (a >= 0 || b >= 0) ? 3 : 2;
    return true;
}

// The packed triangles of leaves lv[0 .. nlv) at tris[at ..]: the caller's
// ids, then their indices and flags, then the vertices, each step's loads
// issued together.
__device__ __forceinline__ void emit_leaf_tris(const BuildArgs &A, const int32_t *lv, int nlv, int32_t at)
{
    int32_t id[kMaxLeafTris];
    int3 t[kMaxLeafTris];
    uint32_t fl[kMaxLeafTris];
#pragma unroll
    for (int j = 0; j < kMaxLeafTris; ++j)
        if (j < nlv) id[j] = A.vals[~lv[j]];
#pragma unroll
    for (int j = 0; j < kMaxLeafTris; ++j)
        if (j < nlv) {
            t[j] = A.idx[id[j]];
            fl[j] = A.flags ? A.flags[id[j]] : 0u;
        }
#pragma unroll
    for (int j = 0; j < kMaxLeafTris; ++j)
        if (j < nlv) {
            const float *v = A.verts;
            PackedTri P;
            P.w0 = make_float4(v[3 * t[j].x], v[3 * t[j].x + 1], v[3 * t[j].x + 2], v[3 * t[j].y]);
            P.w1 = make_float4(v[3 * t[j].y + 1], v[3 * t[j].y + 2], v[3 * t[j].z], v[3 * t[j].z + 1]);
            P.w2 = make_float4(v[3 * t[j].z + 2], __int_as_float(id[j]), __uint_as_float(fl[j]), 0.f);
            A.tris[at + j] = P;
        }
}

// The children of wide node `node` by the surface-area decisions: its 8
// slots split between the binary children, recursively, until a subtree
// gets one slot (a leaf slot or a wide child node).
__device__ __forceinline__ int sah_children(const BuildArgs &A, int32_t node, int32_t *ch, bool *leaf)
{
    int32_t st_ref[8];
    int st_n[8];
    int sp = 0, m = 0;
    const uint32_t d = A.dec[node];
    const int k8 = (int)((d >> 21) & 7u);
    st_ref[sp] = A.right[node]; st_n[sp++] = 8 - k8;
    st_ref[sp] = A.left[node]; st_n[sp++] = k8;
    while (sp > 0 && m < 8) {
        --sp;
        const int32_t r = st_ref[sp];
        int i = st_n[sp];
        if (r < 0) { ch[m] = r; leaf[m] = true; ++m; continue; }
        const uint32_t dr = A.dec[r];
        while (i >= 2 && ((dr >> (3 * (i - 2))) & 7u) == 0u) --i;
        if (i <= 1) {
            ch[m] = r;
            leaf[m] = (dr >> 31) != 0u;
            ++m;
            continue;
        }
        const int k = (int)((dr >> (3 * (i - 2))) & 7u);
        if (sp + 2 > 8) { ch[m] = r; leaf[m] = false; ++m; continue; }   // cannot happen: slots sum to 8
        st_ref[sp] = A.right[r]; st_n[sp++] = i - k;
        st_ref[sp] = A.left[r]; st_n[sp++] = k;
    }
    return m;
}

// One thread per wide node of the current level: gather up to 8 children
// (by the surface-area decisions, or greedily by repeatedly opening the
// largest-area internal child, those too big for a leaf first), assign slots
// by octant, quantise, emit leaves and tasks.
__device__ __forceinline__ void collapse_task(const BuildArgs &A, const int2 task)
{
    const int32_t wide = task.y;

    int32_t ch[8];
    float4 clo[8], chi[8];
    float area[8];
    int32_t cnt[8];
    bool leaf[8];
    int m = 0;
    if (task.x < 0) {
        ch[0] = task.x; m = 1;
    } else if (A.dec) {
        m = sah_children(A, task.x, ch, leaf);
    } else {
        ch[0] = A.left[task.x]; ch[1] = A.right[task.x]; m = 2;
    }
    for (int k = 0; k < m; ++k) {
        ref_box(A, ch[k], clo[k], chi[k]);
        area[k] = half_area(clo[k], chi[k]);
        cnt[k] = ref_count(A, ch[k]);
    }
    while (!A.dec && m < 8) {
        int best = -1;
        float best_a = -1.f;
        for (int pass = 0; pass < 2 && best < 0; ++pass) {
            for (int k = 0; k < m; ++k) {
                if (ch[k] < 0) continue;
                if (pass == 0 && cnt[k] <= kMaxLeafTris) continue;
                if (area[k] > best_a) { best_a = area[k]; best = k; }
            }
        }
        if (best < 0) break;
        const int32_t node = ch[best];
        ch[best] = A.left[node];
        ch[m] = A.right[node];
        ref_box(A, ch[best], clo[best], chi[best]);
        ref_box(A, ch[m], clo[m], chi[m]);
        area[best] = half_area(clo[best], chi[best]);
        area[m] = half_area(clo[m], chi[m]);
        cnt[best] = ref_count(A, ch[best]);
        cnt[m] = ref_count(A, ch[m]);
        ++m;
    }

    if (!A.dec || task.x < 0)
        for (int k = 0; k < m; ++k) leaf[k] = cnt[k] <= kMaxLeafTris;
    for (int k = 0; k < m; ++k)
        if (leaf[k] && cnt[k] > kMaxLeafTris) { atomicExch(&A.counters[3], 1); return; }

    // node box and centroid
    float4 nlo = clo[0], nhi = chi[0];
    for (int k = 1; k < m; ++k) {
        nlo = make_float4(fminf(nlo.x, clo[k].x), fminf(nlo.y, clo[k].y), fminf(nlo.z, clo[k].z), 0.f);
        nhi = make_float4(fmaxf(nhi.x, chi[k].x), fmaxf(nhi.y, chi[k].y), fmaxf(nhi.z, chi[k].z), 0.f);
    }
    const float pcx = 0.5f * (nlo.x + nhi.x), pcy = 0.5f * (nlo.y + nhi.y), pcz = 0.5f * (nlo.z + nhi.z);

    // slot assignment: slot s holds the child met first by rays of octant s
    // (direction signs = bits of s); greedy on dot(centroid offset, signs).
    int slot_of[8];
    int child_in[8];
    for (int s = 0; s < 8; ++s) child_in[s] = -1;
    for (int k = 0; k < m; ++k) slot_of[k] = -1;
    for (int it = 0; it < m; ++it) {
        float bc = FLT_MAX;
        int bk = 0, bs = 0;
        for (int k = 0; k < m; ++k) {
            if (slot_of[k] >= 0) continue;
            const float ox = 0.5f * (clo[k].x + chi[k].x) - pcx;
            const float oy = 0.5f * (clo[k].y + chi[k].y) - pcy;
            const float oz = 0.5f * (clo[k].z + chi[k].z) - pcz;
            for (int s = 0; s < 8; ++s) {
                if (child_in[s] >= 0) continue;
                const float c = ((s & 1) ? -ox : ox) + ((s & 2) ? -oy : oy) + ((s & 4) ? -oz : oz);
                if (c < bc) { bc = c; bk = k; bs = s; }
            }
        }
        slot_of[bk] = bs;
        child_in[bs] = bk;
    }

    // allocate children nodes and triangle slots
    int n_int = 0, n_tri = 0;
    for (int k = 0; k < m; ++k) {
        if (!leaf[k]) ++n_int; else n_tri += cnt[k];
    }
    const unsigned long long old = (n_int || n_tri) ? alloc_nodes_tris(A.counters, n_int, n_tri) : 0ull;
    const int32_t child_base = (int32_t)(uint32_t)old;
    const int32_t tri_base = (int32_t)(old >> 32);
    if (child_base + n_int > A.max_nodes || tri_base + n_tri > A.n) { atomicExch(&A.counters[3], 1); return; }

    // quantisation frame
    const int ex = grid_exponent(nhi.x - nlo.x), ey = grid_exponent(nhi.y - nlo.y), ez = grid_exponent(nhi.z - nlo.z);
    const float ux = __int_as_float(ex << 23), uy = __int_as_float(ey << 23), uz = __int_as_float(ez << 23);
    const float px = __fsub_rd(nlo.x, ux), py = __fsub_rd(nlo.y, uy), pz = __fsub_rd(nlo.z, uz);
    const float ix = __int_as_float((254 - ex) << 23);   // exact 1/unit
    const float iy = __int_as_float((254 - ey) << 23);
    const float iz = __int_as_float((254 - ez) << 23);

    WideNode W;
    W.px = px; W.py = py; W.pz = pz;
    W.ex = (uint8_t)ex; W.ey = (uint8_t)ey; W.ez = (uint8_t)ez;
    W.imask = 0;
    W.child_base = (uint32_t)child_base;
    W.tri_base = (uint32_t)tri_base;
    int int_k = 0, tri_off = 0;
    for (int s = 0; s < 8; ++s) {
        const int k = child_in[s];
        A.slot_ref[8 * (size_t)wide + s] = k < 0 ? kEmptySlot : ch[k];
        if (k < 0) {
            W.meta[s] = 0;
            W.qlo_x[s] = W.qlo_y[s] = W.qlo_z[s] = 255;
            W.qhi_x[s] = W.qhi_y[s] = W.qhi_z[s] = 0;
            continue;
        }
        const auto qlo = [](float c, float p, float inv) {
            const float q = floorf(__fmul_rd(__fsub_rd(c, p), inv)) - 1.0f;
            return (uint8_t)fminf(fmaxf(q, 0.f), 255.f);
        };
        const auto qhi = [](float c, float p, float inv) {
            const float q = ceilf(__fmul_ru(__fsub_ru(c, p), inv)) + 1.0f;
            return (uint8_t)fminf(fmaxf(q, 0.f), 255.f);
        };
        W.qlo_x[s] = qlo(clo[k].x, px, ix); W.qlo_y[s] = qlo(clo[k].y, py, iy); W.qlo_z[s] = qlo(clo[k].z, pz, iz);
        W.qhi_x[s] = qhi(chi[k].x, px, ix); W.qhi_y[s] = qhi(chi[k].y, py, iy); W.qhi_z[s] = qhi(chi[k].z, pz, iz);
        if (!leaf[k]) {
            W.imask |= (uint8_t)(1u << s);
            W.meta[s] = (uint8_t)(0x20 | (24 + s));
            const int slot = atomicAdd(A.next_count, 1);
            A.tasks_out[slot] = make_int2(ch[k], child_base + int_k);
            ++int_k;
        } else {
            const int c = cnt[k];
            W.meta[s] = (uint8_t)((((1u << c) - 1u) << 5) | (uint32_t)tri_off);
            int32_t lv[kMaxLeafTris];
            int nlv = 0;
            if (!leaf_refs(A, ch[k], lv, nlv) || nlv != c) { atomicExch(&A.counters[3], 1); return; }
            emit_leaf_tris(A, lv, nlv, tri_base + tri_off);
            tri_off += c;
        }
    }
    A.nodes[wide] = W;
}

// The quantised box bytes of a child in the node's frame.
__device__ __forceinline__ uint32_t quant_lo(float c, float p, float inv)
{
    const float q = floorf(__fmul_rd(__fsub_rd(c, p), inv)) - 1.0f;
    return (uint32_t)fminf(fmaxf(q, 0.f), 255.f);
}
__device__ __forceinline__ uint32_t quant_hi(float c, float p, float inv)
{
    const float q = ceilf(__fmul_ru(__fsub_ru(c, p), inv)) + 1.0f;
    return (uint32_t)fminf(fmaxf(q, 0.f), 255.f);
}

// Lane groups of 8 within a warp: ballots, reductions and shuffles confined
// to the group (xor shuffles with offsets 4, 2, 1 never leave an aligned
// group of 8).  Every lane of the warp executes each of them.
__device__ __forceinline__ uint32_t gballot(bool p, int gbase)
{
    return (__ballot_sync(0xffffffffu, p) >> gbase) & 0xffu;
}
__device__ __forceinline__ int gmin(int v)
{
    v = min(v, __shfl_xor_sync(0xffffffffu, v, 4));
    v = min(v, __shfl_xor_sync(0xffffffffu, v, 2));
    return min(v, __shfl_xor_sync(0xffffffffu, v, 1));
}
__device__ __forceinline__ int gmax(int v)
{
    v = max(v, __shfl_xor_sync(0xffffffffu, v, 4));
    v = max(v, __shfl_xor_sync(0xffffffffu, v, 2));
    return max(v, __shfl_xor_sync(0xffffffffu, v, 1));
}
__device__ __forceinline__ uint32_t gor(uint32_t v)
{
    v |= __shfl_xor_sync(0xffffffffu, v, 4);
    v |= __shfl_xor_sync(0xffffffffu, v, 2);
    return v | __shfl_xor_sync(0xffffffffu, v, 1);
}

// Word h (0: slots 0-3, 1: slots 4-7) of a per-slot byte plane: every lane
// of the group that holds a child in that half contributes its byte; empty
// slots read `empty`.
__device__ __forceinline__ uint32_t plane_word(bool mine, int slot, uint32_t byte, int h, uint32_t empty)
{
    const bool in = mine && (slot >> 2) == h;
    const uint32_t sh = 8u * (uint32_t)(slot & 3);
    const uint32_t occ = gor(in ? (0xffu << sh) : 0u);
    const uint32_t val = gor(in ? (byte << sh) : 0u);
    return (empty & ~occ) | val;
}

// One wide node per group of 8 lanes (surface-area decisions), four per
// warp: lane k of the group holds child k.  The 8 slots are split between
// binary children in rounds (a lane that splits keeps the left share and
// hands the right one to a new lane), then lanes load their boxes, the node
// box is a group reduction, slots go to children by repeated group arg-min
// of the octant cost, and the node's 20 words are assembled with group OR
// reductions.  Same node as collapse_task up to the order of equal-cost
// choices.  Several nodes per warp keep four times as many of a level's
// dependent-load chains (decisions, children, boxes) in flight as one node
// per warp, on the wide levels near the leaves where a level's tasks far
// outnumber the resident warps.  Control flow stays warp-uniform (groups
// without a task, or with a malformed one, only stop writing).
__device__ __forceinline__ void collapse_task_group(const BuildArgs &A, const int2 task, bool has_task, int gbase,
                                                    int lane)
{
    const uint32_t full = 0xffffffffu;
    int32_t ref = 0;
    int slots = 0;
    bool active = false, done = false, lf = false, err = false;
    if (has_task) {
        if (task.x < 0) {
            if (lane == 0) { ref = task.x; active = done = lf = true; }
        } else {
            const uint32_t d = A.dec[task.x];
            const int k8 = (int)((d >> 21) & 7u);
            if (lane == 0) { ref = A.left[task.x]; slots = k8; active = true; }
            if (lane == 1) { ref = A.right[task.x]; slots = 8 - k8; active = true; }
        }
    }
    for (int round = 0; round < 8; ++round) {
        bool split = false;
        int32_t rr = 0;
        int rs = 0;
        if (active && !done) {
            if (ref < 0) {
                done = lf = true;
            } else {
                // the children are loaded with the decision (one round trip)
                const uint32_t dr = A.dec[ref];
                const int32_t lref = A.left[ref], rref = A.right[ref];
                int i = slots;
                while (i >= 2 && ((dr >> (3 * (i - 2))) & 7u) == 0u) --i;
                if (i <= 1) {
                    done = true;
                    lf = (dr >> 31) != 0u;
                } else {
                    const int kl = (int)((dr >> (3 * (i - 2))) & 7u);
                    split = true;
                    rr = rref;
                    rs = i - kl;
                    ref = lref;
                    slots = kl;
                }
            }
        }
        const uint32_t sb = gballot(split, gbase);
        if (!__any_sync(full, sb != 0u)) break;
        const int nact = __popc(gballot(active, gbase));
        const int nsb = __popc(sb);
        if (nact + nsb > 8) err = true;   // the slot shares always sum to 8
        // receiving lane nact + r takes the right share of the r-th splitter
        const int r = lane - nact;
        const bool recv = !err && r >= 0 && r < nsb;
        const int src = recv ? (int)__fns(sb, 0, r + 1) : lane;
        const int32_t got_ref = __shfl_sync(full, rr, gbase + src);
        const int got_slots = __shfl_sync(full, rs, gbase + src);
        if (recv) {
            ref = got_ref;
            slots = got_slots;
            active = true;
            done = lf = false;
        }
    }
    const int m = __popc(gballot(active, gbase));
    if (gballot(active && !done, gbase) != 0u) err = true;
    if (err) active = false;

    float4 lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
    int32_t cnt = 0;
    if (active) {
        ref_box(A, ref, lo, hi);
        cnt = ref_count(A, ref);
        if (lf && cnt > kMaxLeafTris) lf = false;   // cannot happen: the tables allow <= 3
    }
    // node box
    const float nlox = of_ord(gmin(ord_of(lo.x)));
    const float nloy = of_ord(gmin(ord_of(lo.y)));
    const float nloz = of_ord(gmin(ord_of(lo.z)));
    const float nhix = of_ord(gmax(ord_of(hi.x)));
    const float nhiy = of_ord(gmax(ord_of(hi.y)));
    const float nhiz = of_ord(gmax(ord_of(hi.z)));
    const float pcx = 0.5f * (nlox + nhix), pcy = 0.5f * (nloy + nhiy), pcz = 0.5f * (nloz + nhiz);

    // slots: slot s holds the child met first by rays of octant s
    const float ox = 0.5f * (lo.x + hi.x) - pcx, oy = 0.5f * (lo.y + hi.y) - pcy, oz = 0.5f * (lo.z + hi.z) - pcz;
    int myslot = -1;
    uint32_t taken = 0;
    for (int it = 0; it < 8; ++it) {
        if (!__any_sync(full, it < m)) break;
        const bool open = active && myslot < 0;
        float bc = FLT_MAX;
        int bs = 0;
        if (open) {
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                if ((taken >> s) & 1u) continue;
                const float c = ((s & 1) ? -ox : ox) + ((s & 2) ? -oy : oy) + ((s & 4) ? -oz : oz);
                if (c < bc) { bc = c; bs = s; }
            }
        }
        const int o = open ? ord_of(bc) : 0x7fffffff;
        const int mn = gmin(o);
        const uint32_t cand = gballot(open && o == mn, gbase);
        const int winner = cand ? __ffs(cand) - 1 : 0;
        const int ws = __shfl_sync(full, bs, gbase + winner);
        if (cand) {
            if (lane == winner) myslot = ws;
            taken |= 1u << ws;
        }
    }

    // allocation: internal children contiguous in slot order, leaf triangles
    // in slot order
    const bool internal = active && !lf;
    const uint32_t imask = gor(internal ? (1u << myslot) : 0u);
    const int n_int = __popc(imask);
    const uint32_t cnt_lo = gor((active && lf && myslot < 4) ? ((uint32_t)cnt << (8 * myslot)) : 0u);
    const uint32_t cnt_hi = gor((active && lf && myslot >= 4) ? ((uint32_t)cnt << (8 * (myslot - 4))) : 0u);
    int n_tri = 0, tri_off = 0;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int c = (int)(((s < 4 ? cnt_lo : cnt_hi) >> (8 * (s & 3))) & 0xffu);
        if (s < myslot) tri_off += c;
        n_tri += c;
    }
    const bool writes = has_task && !err;
    // allocation for the warp's four tasks at once: one atomic per counter
    // (every task of a level adds to the same three addresses)
    int32_t child_base = 0, tri_base = 0, next = 0;
    {
        const int mi = writes ? n_int : 0, mt = writes ? n_tri : 0;
        int pi = 0, pt = 0, si = 0, st = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int vi = __shfl_sync(full, mi, 8 * q), vt = __shfl_sync(full, mt, 8 * q);
            if (8 * q < gbase) { pi += vi; pt += vt; }
            si += vi;
            st += vt;
        }
        int32_t cb = 0, tb = 0, nb = 0;
        if ((threadIdx.x & 31) == 0) {
            if (si || st) {
                const unsigned long long old = alloc_nodes_tris(A.counters, si, st);
                cb = (int32_t)(uint32_t)old;
                tb = (int32_t)(old >> 32);
            }
            if (si) nb = atomicAdd(A.next_count, si);
        }
        child_base = __shfl_sync(full, cb, 0) + pi;
        tri_base = __shfl_sync(full, tb, 0) + pt;
        next = __shfl_sync(full, nb, 0) + pi;
    }
    const bool fits = child_base + n_int <= A.max_nodes && tri_base + n_tri <= A.n;
    if (has_task && lane == 0 && (err || !fits)) atomicExch(&A.counters[3], 1);
    if (!writes || !fits) active = false;

    // quantisation frame
    const int ex = grid_exponent(nhix - nlox), ey = grid_exponent(nhiy - nloy), ez = grid_exponent(nhiz - nloz);
    const float ux = __int_as_float(ex << 23), uy = __int_as_float(ey << 23), uz = __int_as_float(ez << 23);
    const float px = __fsub_rd(nlox, ux), py = __fsub_rd(nloy, uy), pz = __fsub_rd(nloz, uz);
    const float ix = __int_as_float((254 - ex) << 23);   // exact 1/unit
    const float iy = __int_as_float((254 - ey) << 23);
    const float iz = __int_as_float((254 - ez) << 23);
    uint32_t meta = 0, qlx = 255, qly = 255, qlz = 255, qhx = 0, qhy = 0, qhz = 0;
    if (active) {
        qlx = quant_lo(lo.x, px, ix); qly = quant_lo(lo.y, py, iy); qlz = quant_lo(lo.z, pz, iz);
        qhx = quant_hi(hi.x, px, ix); qhy = quant_hi(hi.y, py, iy); qhz = quant_hi(hi.z, pz, iz);
        meta = internal ? (0x20u | (uint32_t)(24 + myslot)) : ((((1u << cnt) - 1u) << 5) | (uint32_t)tri_off);
    }
    uint32_t w[20];
    w[0] = __float_as_uint(px);
    w[1] = __float_as_uint(py);
    w[2] = __float_as_uint(pz);
    w[3] = (uint32_t)ex | ((uint32_t)ey << 8) | ((uint32_t)ez << 16) | (imask << 24);
    w[4] = (uint32_t)child_base;
    w[5] = (uint32_t)tri_base;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        w[6 + h] = plane_word(active, myslot, meta, h, 0u);
        w[8 + h] = plane_word(active, myslot, qlx, h, 0xffffffffu);
        w[10 + h] = plane_word(active, myslot, qly, h, 0xffffffffu);
        w[12 + h] = plane_word(active, myslot, qlz, h, 0xffffffffu);
        w[14 + h] = plane_word(active, myslot, qhx, h, 0u);
        w[16 + h] = plane_word(active, myslot, qhy, h, 0u);
        w[18 + h] = plane_word(active, myslot, qhz, h, 0u);
    }
    const uint32_t occ = gor(active ? (1u << myslot) : 0u);
    if (!writes || !fits) return;   // after the last group operation
    if (lane < 5) {
        uint4 v;
        v.x = w[0]; v.y = w[1]; v.z = w[2]; v.w = w[3];
#pragma unroll
        for (int q = 1; q < 5; ++q)
            if (lane == q) { v.x = w[4 * q]; v.y = w[4 * q + 1]; v.z = w[4 * q + 2]; v.w = w[4 * q + 3]; }
        reinterpret_cast<uint4 *>(A.nodes + task.y)[lane] = v;
    }
    if (active) A.slot_ref[8 * (size_t)task.y + myslot] = ref;
    if (!((occ >> lane) & 1u)) A.slot_ref[8 * (size_t)task.y + lane] = kEmptySlot;
    if (internal) {
        const int rank = __popc(imask & ((1u << myslot) - 1u));
        A.tasks_out[next + rank] = make_int2(ref, child_base + rank);
    } else if (active) {
        int32_t lv[kMaxLeafTris];
        int nlv = 0;
        if (!leaf_refs(A, ref, lv, nlv) || nlv != cnt) {
            atomicExch(&A.counters[3], 1);
            return;
        }
        emit_leaf_tris(A, lv, nlv, tri_base + tri_off);
    }
}

// 10 resident blocks (48 registers): the level launches are bound by the
// latency of each task's chain of dependent loads, so resident warps count
// for more than the registers that keep the leaf loads in flight together
#ifndef RT_COLLAPSE_MIN_BLOCKS
#define RT_COLLAPSE_MIN_BLOCKS 10
#endif
__global__ void __launch_bounds__(128, RT_COLLAPSE_MIN_BLOCKS) k_collapse_level_group(BuildArgs A)
{
    const int32_t ntasks = *A.cur_count;
    const int lane32 = threadIdx.x & 31;
    const int g = lane32 >> 3;
    const int32_t wid = (int32_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int32_t nw = (int32_t)((gridDim.x * blockDim.x) >> 5);
    for (int32_t t0 = 4 * wid; t0 < ntasks; t0 += 4 * nw) {
        const int32_t ti = t0 + g;
        const bool has = ti < ntasks;
        collapse_task_group(A, has ? A.tasks_in[ti] : make_int2(0, 0), has, 8 * g, lane32 & 7);
    }
}

// The first kCollapseTopLevels levels of a single-root tree (at most 1, 8
// and 64 tasks) in one block, between block barriers: the levels near the
// root are a chain of dependent loads per task, and one launch for all
// three saves two launches' fixed cost.
constexpr int kCollapseTopLevels = 3;
__global__ void __launch_bounds__(1024) k_collapse_top(BuildArgs A, int2 *tq0, int2 *tq1, int32_t *level_count)
{
    const int lane32 = threadIdx.x & 31;
    const int g = lane32 >> 3;
    const int32_t wid = (int32_t)(threadIdx.x >> 5);
    const int32_t nw = (int32_t)(blockDim.x >> 5);
    for (int level = 0; level < kCollapseTopLevels; ++level) {
        BuildArgs B = A;
        B.tasks_in = (level & 1) ? tq1 : tq0;
        B.tasks_out = (level & 1) ? tq0 : tq1;
        B.cur_count = level_count + level;
        B.next_count = level_count + level + 1;
        const int32_t ntasks = __ldcg(B.cur_count);   // counted by this block's previous level
        for (int32_t t0 = 4 * wid; t0 < ntasks; t0 += 4 * nw) {
            const int32_t ti = t0 + g;
            const bool has = ti < ntasks;
            collapse_task_group(B, has ? __ldcg(B.tasks_in + ti) : make_int2(0, 0), has, 8 * g, lane32 & 7);
        }
        __syncthreads();
    }
}

// One tree level: every task of the level (count read on the device, so
// the levels run back to back without host round trips).
__global__ void k_collapse_level(BuildArgs A)
{
    const int32_t ntasks = *A.cur_count;
    for (int32_t ti = blockIdx.x * blockDim.x + threadIdx.x; ti < ntasks; ti += gridDim.x * blockDim.x)
        collapse_task(A, A.tasks_in[ti]);
}

}  // namespace

size_t build_temp_bytes(int32_t n)
{
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, (const uint64_t *)nullptr, (uint64_t *)nullptr,
                                    (const int32_t *)nullptr, (int32_t *)nullptr, n > 0 ? n : 1, 0, 64);
    const size_t nn = (size_t)(n > 0 ? n : 1);
    size_t b = 0;
    b += 2 * nn * sizeof(float4);          // blo, bhi
    b += 2 * nn * sizeof(uint64_t);        // keys in/out
    b += 2 * nn * sizeof(int32_t);         // vals in/out
    b += 6 * nn * sizeof(int32_t);         // left right first last parent leaf_parent
    b += 4 * nn * sizeof(float4);          // llo lhi ilo ihi
    b += nn * sizeof(int32_t);             // refit flags
    b += 2 * nn * sizeof(int2);            // task queues
    b += nn * sizeof(int32_t);             // leaf counts of internal nodes
    b += 8 * (nn + kMaxSegments + 2) * sizeof(int32_t);   // slot refs of the wide nodes
    b += 9 * nn * sizeof(float);           // surface-area cost tables + decisions
    b += 4 * nn * sizeof(float4);          // PLOC clusters (two buffers of lo, hi)
    b += nn * sizeof(int32_t);             // PLOC nearest neighbours
    b += (nn / kPlocBlock + 2) * sizeof(int2) + kStWords * sizeof(int32_t);
    b += 16 * sizeof(int32_t) + 2 * nn * sizeof(int2);   // counters, root tasks
    b += (6 + 1) * (size_t)kMaxSegments * sizeof(int) + 1024;
    b += cub_bytes + 16 * 256;
    return b;
}

static inline char *carve(char *&p, size_t bytes)
{
    char *r = p;
    p += (bytes + 255) & ~(size_t)255;
    return r;
}

BuildResult build_wide_bvh(const BuildInputs &in, void *temp, size_t temp_bytes, cudaStream_t st)
{
    BuildResult R;
    const int32_t n = in.ntris;
    const int32_t nseg = in.nseg > 0 ? in.nseg : 1;
    if (nseg > kMaxSegments) { R.status = -1; return R; }
    if (n <= 0 && nseg == 1) { R.status = 0; return R; }
    const size_t nn = (size_t)(n > 0 ? n : 1);
    char *p = (char *)temp;
    float4 *blo = (float4 *)carve(p, nn * sizeof(float4));
    float4 *bhi = (float4 *)carve(p, nn * sizeof(float4));
    uint64_t *keys = (uint64_t *)carve(p, nn * sizeof(uint64_t));
    uint64_t *keys2 = (uint64_t *)carve(p, nn * sizeof(uint64_t));
    int32_t *vals = (int32_t *)carve(p, nn * sizeof(int32_t));
    int32_t *vals2 = (int32_t *)carve(p, nn * sizeof(int32_t));
    int32_t *left = (int32_t *)carve(p, nn * sizeof(int32_t));
    int32_t *right = (int32_t *)carve(p, nn * sizeof(int32_t));
    int32_t *first = (int32_t *)carve(p, nn * sizeof(int32_t));
    int32_t *last = (int32_t *)carve(p, nn * sizeof(int32_t));
    int32_t *parent = (int32_t *)carve(p, nn * sizeof(int32_t));
    int32_t *leaf_parent = (int32_t *)carve(p, nn * sizeof(int32_t));
    float4 *llo = (float4 *)carve(p, nn * sizeof(float4));
    float4 *lhi = (float4 *)carve(p, nn * sizeof(float4));
    float4 *ilo = (float4 *)carve(p, nn * sizeof(float4));
    float4 *ihi = (float4 *)carve(p, nn * sizeof(float4));
    int32_t *rflags = (int32_t *)carve(p, nn * sizeof(int32_t));
    int32_t *ncount = (int32_t *)carve(p, nn * sizeof(int32_t));
    int32_t *slot_ref = (int32_t *)carve(p, 8 * ((size_t)in.max_nodes + 1) * sizeof(int32_t));
    float *sah = RT_COLLAPSE_SAH ? (float *)carve(p, 8 * nn * sizeof(float)) : nullptr;
    uint32_t *dec = RT_COLLAPSE_SAH ? (uint32_t *)carve(p, nn * sizeof(uint32_t)) : nullptr;
    const bool ploc = in.builder == kBuilderPloc || in.builder == kBuilderHploc;
    const bool hploc = in.builder == kBuilderHploc && nseg == 1;   // batches cluster with PLOC
    float4 *cl[2] = {nullptr, nullptr}, *chh[2] = {nullptr, nullptr};
    int32_t *nnb = nullptr, *pstate = nullptr;
    unsigned long long *meet = nullptr;
    int32_t *cref = nullptr;
    int2 *bsum = nullptr;
    if (ploc) {
        cl[0] = (float4 *)carve(p, nn * sizeof(float4));
        chh[0] = (float4 *)carve(p, nn * sizeof(float4));
        cl[1] = (float4 *)carve(p, nn * sizeof(float4));
        chh[1] = (float4 *)carve(p, nn * sizeof(float4));
        nnb = (int32_t *)carve(p, nn * sizeof(int32_t));
        if (hploc) {
            meet = (unsigned long long *)carve(p, nn * sizeof(unsigned long long));
            cref = (int32_t *)carve(p, nn * sizeof(int32_t));
        }
        bsum = (int2 *)carve(p, (nn / kPlocBlock + 2) * sizeof(int2));
        pstate = (int32_t *)carve(p, kStWords * sizeof(int32_t));
    }
    int2 *tq0 = (int2 *)carve(p, (nn + nseg) * sizeof(int2));
    int2 *tq1 = (int2 *)carve(p, (nn + nseg) * sizeof(int2));
    int32_t *counters = (int32_t *)carve(p, 16 * sizeof(int32_t));
    int32_t *level_count = (int32_t *)carve(p, (kMaxDepth + 2) * sizeof(int32_t));
    int *cbounds = (int *)carve(p, 6 * (size_t)nseg * sizeof(int));
    int32_t *seg_first = (int32_t *)carve(p, ((size_t)nseg + 1) * sizeof(int32_t));
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, keys, keys2, vals, vals2, (int)nn, 0, 64, st);
    void *cub_temp = carve(p, cub_bytes);
    if ((size_t)(p - (char *)temp) > temp_bytes) { R.status = -3; return R; }

    // segment offsets (sorted positions of each segment = its triangle range)
    int32_t *h_cnt = in.host_scratch;   // pinned, >= 6 + kMaxDepth ints
    std::vector<int> init_bounds(6 * (size_t)nseg);
    for (int s = 0; s < nseg; ++s)
        for (int k = 0; k < 3; ++k) { init_bounds[6 * s + k] = 0x7fffffff; init_bounds[6 * s + 3 + k] = (int)0x80000000; }
    cudaMemsetAsync(counters, 0, 16 * sizeof(int32_t), st);
    cudaMemcpyAsync(cbounds, init_bounds.data(), init_bounds.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    if (nseg > 1) {
        cudaMemcpyAsync(seg_first, in.seg_first, ((size_t)nseg + 1) * sizeof(int32_t), cudaMemcpyDefault, st);
    } else {
        const int32_t sf[2] = {0, n};
        cudaMemcpyAsync(seg_first, sf, sizeof(sf), cudaMemcpyHostToDevice, st);
    }
    int sb = 0;
    while ((1 << sb) < nseg) ++sb;
    // Morton bits per axis: as asked; else, from a million triangles up,
    // about log2(n) / 3 + 3 (cells of a few triangles at most, so the order
    // the builders start from keeps neighbours together, in fewer radix
    // passes); below that the sort costs little and the full width keeps
    // small meshes' finer order (20k-triangle icosphere: 0.116 ms per frame
    // against 0.127 ms at 10 bits); never more than the key holds
    int lg = 0;
    while (lg < 31 && (1 << lg) < n) ++lg;
    int mbits = in.morton_bits > 0 ? in.morton_bits : (n < (1 << 20) ? 21 : (lg + 2) / 3 + 3);
    mbits = max(10, min(mbits, (63 - sb) / 3));
    const int key_bits = 3 * mbits + sb;
    const int threads = 256;
    if (n > 0) {
        const int grid_pts = min((n + threads - 1) / threads, in.sm_count * 8);
        k_prep<<<grid_pts, threads, 0, st>>>(in.verts, in.idx, n, in.seg_of_tri, nseg, in.shade, blo, bhi, cbounds);
        k_morton<<<grid_pts, threads, 0, st>>>(blo, bhi, n, in.seg_of_tri, nseg, mbits, cbounds, keys, vals);
        cub::DeviceRadixSort::SortPairs(cub_temp, cub_bytes, keys, keys2, vals, vals2, n, 0, key_bits, st);
        const int g = (n + threads - 1) / threads;
        k_leaf_boxes<<<g, threads, 0, st>>>(vals2, n, blo, bhi, llo, lhi);
        if (!ploc) {
            if (n > 1) k_karras<<<g, threads, 0, st>>>(keys2, n, left, right, first, last, ncount, parent, leaf_parent);
            if (n > 1) {
                cudaMemsetAsync(rflags, 0, nn * sizeof(int32_t), st);
                k_refit<<<g, threads, 0, st>>>(n, left, right, parent, leaf_parent, llo, lhi, ilo, ihi, rflags,
                                               ncount, sah, dec, counters + 3);
            }
        }
    }
    // segment roots -> level-0 tasks (counted in level_count[0]); wide nodes
    // 0..nseg-1 are the roots
    cudaMemsetAsync(level_count, 0, (kMaxDepth + 2) * sizeof(int32_t), st);
    if (ploc) {
        cudaMemsetAsync(pstate, 0, kStWords * sizeof(int32_t), st);
        k_ploc_segments<<<(nseg + 127) / 128, 128, 0, st>>>(nseg, n, seg_first, pstate, in.nodes);
        if (n > 0 && (!hploc || n == 1))
            k_ploc_init<<<min((n + threads - 1) / threads, in.sm_count * 8), threads, 0, st>>>(
                n, keys2, 3 * mbits, nseg, llo, lhi, cl[0], chh[0]);
        // iterations in groups of kPlocGroup, then one read-back of the count
        const int tiles = (n + kPlocTile - 1) / kPlocTile;
        const int blocks = (n + kPlocBlock - 1) / kPlocBlock;
        int it = 0;
        bool finished = n <= 0;
        const size_t tail_smem = 2 * kPlocTailMax * sizeof(float4) + kPlocTailMax * sizeof(int32_t);
        if (cudaFuncSetAttribute(k_ploc_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tail_smem) !=
            cudaSuccess) { R.status = -2; return R; }
        bool tail = !finished && n <= kPlocTailMax && !hploc;
        if (hploc && !finished) {
            k_hploc_init<<<min((n + threads - 1) / threads, in.sm_count * 8), threads, 0, st>>>(n, meet);
            k_hploc<<<(n + kHplocBlock - 1) / kHplocBlock, kHplocBlock, 0, st>>>(
                n, keys2, cref, meet, pstate, llo, lhi, cl[0], chh[0], left, right, ncount, ilo, ihi, sah, dec,
                parent, leaf_parent);
            finished = true;
        }
        while (!finished && !tail) {
            for (int k = 0; k < kPlocGroup; ++k, ++it) {
                const int a = it & 1;
                k_ploc_nn<<<max(tiles, 1), kPlocTile, 0, st>>>(cl[a], chh[a], nnb, pstate, it);
                k_ploc_count<<<max(blocks, 1), kPlocBlock, 0, st>>>(nnb, pstate, it, bsum);
                k_ploc_scan<<<1, kPlocBlock, 0, st>>>(bsum, pstate, it);
                k_ploc_merge<<<max(blocks, 1), kPlocBlock, 0, st>>>(cl[a], chh[a], cl[a ^ 1], chh[a ^ 1], nnb, bsum,
                                                                    pstate, it, left, right, ncount, ilo, ihi,
                                                                    sah, dec, parent, leaf_parent);
            }
            cudaMemcpyAsync(h_cnt, pstate, kStWords * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) { R.status = -2; return R; }
            if (h_cnt[kStError]) { R.status = -6; return R; }
            finished = h_cnt[kStCount + (it & 1)] <= h_cnt[kStTarget];
            tail = !finished && h_cnt[kStCount + (it & 1)] <= kPlocTailMax;
            if (!finished && !tail && it >= kPlocMaxIterations) { R.status = -6; return R; }
        }
        if (tail)
            k_ploc_tail<<<1, kPlocBlock, tail_smem, st>>>(cl[it & 1], chh[it & 1], pstate, it, left, right, ncount,
                                                          ilo, ihi, sah, dec, parent, leaf_parent);
        k_ploc_roots<<<(nseg + 127) / 128, 128, 0, st>>>(cl[it & 1], chh[it & 1], pstate, it, tq0, level_count,
                                                        counters, parent, leaf_parent);
    } else {
        k_roots<<<(nseg + 127) / 128, 128, 0, st>>>(nseg, n, seg_first, first, last, parent, leaf_parent, tq0,
                                                    level_count, counters, in.nodes);
    }
    const int32_t nroot_nodes = nseg;
    cudaMemcpyAsync(&counters[0], &nroot_nodes, sizeof(int32_t), cudaMemcpyHostToDevice, st);

    BuildArgs A;
    A.n = n; A.left = left; A.right = right; A.count = ncount; A.dec = dec; A.slot_ref = slot_ref;
    A.ilo = ilo; A.ihi = ihi; A.llo = llo; A.lhi = lhi; A.vals = vals2;
    A.verts = in.verts; A.idx = in.idx; A.flags = in.flags;
    A.nodes = in.nodes; A.tris = in.tris; A.counters = counters;
    A.max_nodes = in.max_nodes;
    int depth = 0;
    // levels back to back in groups of kCollapseGroup (a level past the last
    // one finds no tasks), one read-back per group: most trees end within
    // the first group; a single root's first levels in one block
    const int cgrid = max(1, min((n + nseg + 63) / 64, in.sm_count * 16));
    const int wgrid = max(1, min((n + nseg + 3) / 4, in.sm_count * 32));
    int level = 0;
    if (A.dec && nseg == 1) {
        k_collapse_top<<<1, 1024, 0, st>>>(A, tq0, tq1, level_count);
        level = kCollapseTopLevels;
    }
    for (bool first = true;; first = false) {
        // the first group ends at level kCollapseGroup whichever level it starts at
        const int stop = min(first ? max(level + 1, kCollapseGroup) : level + kCollapseGroup, kMaxDepth);
        for (; level < stop; ++level) {
            A.tasks_in = (level & 1) ? tq1 : tq0;
            A.tasks_out = (level & 1) ? tq0 : tq1;
            A.cur_count = level_count + level;
            A.next_count = level_count + level + 1;
            if (A.dec)
                k_collapse_level_group<<<wgrid, 128, 0, st>>>(A);
            else
                k_collapse_level<<<cgrid, 64, 0, st>>>(A);
        }
        cudaMemcpyAsync(h_cnt, counters, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(h_cnt + 4, level_count, (kMaxDepth + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        // the clustering's error word (the in-block tail's iteration cap),
        // read with the first group of levels
        if (ploc) cudaMemcpyAsync(h_cnt + 5 + kMaxDepth, pstate + kStError, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { R.status = -2; return R; }
        if (ploc && h_cnt[5 + kMaxDepth]) { R.status = -6; return R; }
        if (level >= kMaxDepth || h_cnt[4 + level] == 0 || h_cnt[3]) break;
    }
    if (h_cnt[3]) { R.status = -8; return R; }
    if (h_cnt[4 + kMaxDepth] != 0) { R.status = -5; return R; }   // deeper than kMaxDepth levels
    while (depth < kMaxDepth && h_cnt[4 + depth] > 0) ++depth;
    R.status = 0;
    R.nodes = h_cnt[0];
    R.tri_slots = h_cnt[1];
    R.depth = depth;
    RefitArrays &K = R.refit;
    K.valid = nseg == 1 && n > 1;
    K.vals = vals2; K.left = left; K.right = right; K.parent = parent; K.leaf_parent = leaf_parent;
    K.blo = blo; K.bhi = bhi; K.llo = llo; K.lhi = lhi; K.ilo = ilo; K.ihi = ihi; K.flags = rflags;
    K.slot_ref = slot_ref; K.err = counters + 3;
    K.ntris = n; K.nnodes = R.nodes; K.tri_slots = R.tri_slots;
    return R;
}

namespace {

// Refit, per triangle (caller's order): shading record and box.
__global__ void k_refit_tris(const float *__restrict__ verts, const int3 *__restrict__ idx, int32_t n,
                             ShadeTri *__restrict__ shade, float4 *__restrict__ blo, float4 *__restrict__ bhi)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int3 t = idx[i];
        const float3 a = make_float3(verts[3 * t.x], verts[3 * t.x + 1], verts[3 * t.x + 2]);
        const float3 b = make_float3(verts[3 * t.y], verts[3 * t.y + 1], verts[3 * t.y + 2]);
        const float3 c = make_float3(verts[3 * t.z], verts[3 * t.z + 1], verts[3 * t.z + 2]);
        const float3 nn = xnorm(xcross(xsub3(b, a), xsub3(c, a)));
        ShadeTri st;
        st.n_cx = make_float4(nn.x, nn.y, nn.z, c.x);
        st.c_yz = make_float2(c.y, c.z);
        st.pad = make_float2(0.f, 0.f);
        shade[i] = st;
        blo[i] = make_float4(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)), 0.f);
        bhi[i] = make_float4(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)), 0.f);
    }
}

// Refit, per wide node: new quantisation frame from its children's refitted
// boxes, every occupied slot re-quantised; links and triangle groups kept.
__global__ void k_requant(WideNode *__restrict__ nodes, int32_t nnodes, const int32_t *__restrict__ slot_ref,
                          const float4 *__restrict__ llo, const float4 *__restrict__ lhi,
                          const float4 *__restrict__ ilo, const float4 *__restrict__ ihi)
{
    const int32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nnodes) return;
    float4 lo[8], hi[8];
    float4 nlo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), nhi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
    uint32_t occ = 0;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int32_t r = slot_ref[8 * (size_t)w + s];
        if (r == kEmptySlot) continue;
        occ |= 1u << s;
        lo[s] = r < 0 ? llo[~r] : __ldcg(&ilo[r]);
        hi[s] = r < 0 ? lhi[~r] : __ldcg(&ihi[r]);
        nlo = make_float4(fminf(nlo.x, lo[s].x), fminf(nlo.y, lo[s].y), fminf(nlo.z, lo[s].z), 0.f);
        nhi = make_float4(fmaxf(nhi.x, hi[s].x), fmaxf(nhi.y, hi[s].y), fmaxf(nhi.z, hi[s].z), 0.f);
    }
    if (!occ) return;
    const int ex = grid_exponent(nhi.x - nlo.x), ey = grid_exponent(nhi.y - nlo.y), ez = grid_exponent(nhi.z - nlo.z);
    const float ux = __int_as_float(ex << 23), uy = __int_as_float(ey << 23), uz = __int_as_float(ez << 23);
    const float px = __fsub_rd(nlo.x, ux), py = __fsub_rd(nlo.y, uy), pz = __fsub_rd(nlo.z, uz);
    const float ix = __int_as_float((254 - ex) << 23);
    const float iy = __int_as_float((254 - ey) << 23);
    const float iz = __int_as_float((254 - ez) << 23);
    WideNode W = nodes[w];
    W.px = px; W.py = py; W.pz = pz;
    W.ex = (uint8_t)ex; W.ey = (uint8_t)ey; W.ez = (uint8_t)ez;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        if (!((occ >> s) & 1u)) continue;
        W.qlo_x[s] = (uint8_t)quant_lo(lo[s].x, px, ix); W.qlo_y[s] = (uint8_t)quant_lo(lo[s].y, py, iy);
        W.qlo_z[s] = (uint8_t)quant_lo(lo[s].z, pz, iz);
        W.qhi_x[s] = (uint8_t)quant_hi(hi[s].x, px, ix); W.qhi_y[s] = (uint8_t)quant_hi(hi[s].y, py, iy);
        W.qhi_z[s] = (uint8_t)quant_hi(hi[s].z, pz, iz);
    }
    nodes[w] = W;
}

// Refit, per packed triangle (leaf order): the new vertices, id and flags kept.
__global__ void k_repack(PackedTri *__restrict__ tris, int32_t nslots, const float *__restrict__ verts,
                         const int3 *__restrict__ idx)
{
    const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nslots) return;
    PackedTri P = tris[j];
    const int3 t = idx[__float_as_int(P.w2.y)];
    P.w0 = make_float4(verts[3 * t.x], verts[3 * t.x + 1], verts[3 * t.x + 2], verts[3 * t.y]);
    P.w1 = make_float4(verts[3 * t.y + 1], verts[3 * t.y + 2], verts[3 * t.z], verts[3 * t.z + 1]);
    P.w2.x = verts[3 * t.z + 2];
    tris[j] = P;
}

}  // namespace

int32_t refit_wide_bvh(const RefitArrays &K, const float *verts, const int3 *idx, ShadeTri *shade, WideNode *nodes,
                       PackedTri *tris, int32_t *host_scratch, cudaStream_t st)
{
    if (!K.valid) return -4;
    const int threads = 256;
    const int32_t n = K.ntris;
    const int g = (n + threads - 1) / threads;
    cudaMemsetAsync(K.err, 0, sizeof(int32_t), st);
    k_refit_tris<<<g, threads, 0, st>>>(verts, idx, n, shade, K.blo, K.bhi);
    k_leaf_boxes<<<g, threads, 0, st>>>(K.vals, n, K.blo, K.bhi, K.llo, K.lhi);
    cudaMemsetAsync(K.flags, 0, (size_t)n * sizeof(int32_t), st);
    k_refit<<<g, threads, 0, st>>>(n, K.left, K.right, K.parent, K.leaf_parent, K.llo, K.lhi, K.ilo, K.ihi, K.flags,
                                   nullptr, nullptr, nullptr, K.err);
    k_requant<<<(K.nnodes + 127) / 128, 128, 0, st>>>(nodes, K.nnodes, K.slot_ref, K.llo, K.lhi, K.ilo, K.ihi);
    k_repack<<<(K.tri_slots + 255) / 256, 256, 0, st>>>(tris, K.tri_slots, verts, idx);
    cudaMemcpyAsync(host_scratch, K.err, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -2;
    return host_scratch[0] ? -8 : 0;
}

}  // namespace rtc
