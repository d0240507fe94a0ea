/*
 * rtcore.h -- C ABI of the GB300 ray-tracing core (sm_103a).
 *
 * Drop-in replacement for the hot path of RAPTor's raytracer/ subsystem:
 * acceleration-structure build, closest-hit / any-hit traversal with
 * Moller-Trumbore triangle tests, and the Phong primary+shadow shading pass.
 * Each entry point names the reference interface it replaces (paths relative
 * to the RAPTor project root).
 *
 * Conventions
 *  - Every function returns rt_status: RT_OK (0) or a negative error code;
 *    nothing aborts.  rt_last_error_string() describes the last error of the
 *    calling thread.
 *  - Pointers to bulk data may be host memory (pageable or pinned) or device
 *    memory of the context's GPU; the core detects which.  Host buffers are
 *    borrowed for the duration of the call; results are complete when the
 *    call returns (host outputs) or when the context's stream reaches the end
 *    of the call's work (device outputs).
 *  - A context owns all device memory it allocates and one CUDA stream
 *    (replaceable with rt_ctx_set_stream).  Calls on one context must not
 *    run concurrently from several threads; distinct contexts are independent.
 *  - Triangle ids are the caller's order (the reference's
 *    primitive_store::indirection ids).  Barycentrics follow the reference:
 *    u weighs vertex c, v weighs vertex b (triangle.h:190-235).
 *  - Arithmetic on the hit path is IEEE binary32 in the reference's
 *    operation order, so hit ids and distances equal the reference's
 *    bit for bit wherever the closest hit is unique.
 */
#ifndef RTCORE_H
#define RTCORE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t rt_status;
#define RT_OK 0
#define RT_ERR_INVALID_ARG (-1)
#define RT_ERR_CUDA (-2)
#define RT_ERR_OUT_OF_MEMORY (-3)
#define RT_ERR_NOT_BUILT (-4)
#define RT_ERR_STACK_OVERFLOW (-5)   /* traversal stack cap hit; results incomplete */
#define RT_ERR_LIMIT (-6)            /* a bounded device loop hit its iteration cap */
#define RT_ERR_NO_DEVICE (-7)
#define RT_ERR_INTERNAL (-8)

typedef struct rt_context rt_context;
typedef struct rt_scene rt_scene;

/* Ray: origin, direction (need not be unit), and the far limit used by
 * any-hit queries (ignored by closest-hit).  32 bytes. */
typedef struct rt_ray {
    float ox, oy, oz, tmax;
    float dx, dy, dz, pad;
} rt_ray;

/* Closest hit: tri = -1 and t = FLT_MAX on a miss (the reference's
 * hit_description with MAX_DIST, common/common.h:230-239). */
typedef struct rt_hit {
    int32_t tri;
    float t, u, v;
} rt_hit;

/* Pinhole camera, exactly the reference camera's constructor arguments
 * (raytracer/camera.h:55-62): position, x/y/z axes, background colour
 * (0..255), half-width w, half-height h, image-plane distance t, resolution.
 * Pixel (x, y) looks along x_axis*(x*2w/xres - w) + y_axis*(y*2h/yres - h)
 * + z_axis*t; row y = 0 is the bottom row (camera.h:127-140). */
typedef struct rt_camera {
    float pos[3];
    float x_axis[3], y_axis[3], z_axis[3];
    float background[3];
    float w, h, t;
    int32_t xres, yres;
} rt_camera;

/* Light (raytracer/light.h:17-34).  kind RT_LIGHT_POINT: point light at pos
 * (spherical light with soft shadows off); RT_LIGHT_DIRECTIONAL: light along
 * dir; RT_LIGHT_SPOT: point light at pos whose intensity falls off with the
 * angle a = acos(shadow-ray direction . dir) as clamp(1 - (a - s_a) /
 * (s_b - s_a), 0, 1) (the spot-light constructor and get_light_intensity,
 * light.h:24-25, 44-59; with s_b = 0 it is a directional light along dir,
 * as light::find_rays treats it, light.h:65).  rgb in 0..255, d the distance
 * drop-off. */
#define RT_LIGHT_POINT 0
#define RT_LIGHT_DIRECTIONAL 1
#define RT_LIGHT_SPOT 2
/* OR-ed into kind: rgb is already divided by 255 -- the colour exactly as
 * the reference's light stores it (light.h:17-34 keep rgb / 255.0f) --
 * and is used as given. */
#define RT_LIGHT_UNIT_RGB 0x100
typedef struct rt_light {
    int32_t kind;
    float rgb[3];
    float pos[3];
    float dir[3];
    float d;
    float s_a, s_b;   /* RT_LIGHT_SPOT: inner and outer cone angles (radians) */
} rt_light;

/* Coloured Phong material (materials/coloured_mapper_shader.h): ka, kd, ks in
 * 0..255, ns the specular exponent.  With per-vertex attributes uploaded, kd
 * is modulated by the barycentric attribute (a per-vertex colour in 0..1).
 * rf: mirror reflectivity (the shader's rf, 0 = none): rt_render adds rf
 * times the colour of the mirror ray (ray::reflect, ray.cc:118-135),
 * recursively while the ray's power (product of rf) exceeds 0.1
 * (MIN_REFLECTIVE_POWER, common.h:31).  A pixel's ray tree (mirror and
 * refracted rays) may be at most RT_MAX_BOUNCES levels below the camera ray
 * and hold at most RT_MAX_TREE_RAYS rays, bounded from the largest rf and
 * tran of the materials in use (worst-case powers rf^i * tran^j above 0.1);
 * materials needing more are refused. */
#define RT_MAX_BOUNCES 31
#define RT_MAX_TREE_RAYS 1024
typedef struct rt_material {
    float ka[3], kd[3], ks[3];
    float ns;
    float rf;
    /* tran: transparency, the weight of the refracted colour (the shader's
     * tran, 0 = opaque); ri: refractive index (inverted for a ray entering
     * the front face).  rt_render adds tran times the colour of the ray of
     * ray::refract (ray.cc:198-281) while its power exceeds 0.1; none beyond
     * the critical angle.  Triangles of a refracting material should carry
     * RT_TRI_TRANSPARENT, as the reference's transparent materials do, so
     * that shadow rays pass them. */
    float tran, ri;
    uint32_t flags;   /* RT_MAT_NO_VERTEX_COLOUR: kd ignores the vertex attribute */
    /* rfd, td: spread of a diffuse reflection and refraction (the shader's
     * rfd and td, coloured_mapper_shader.h:21-22; 0 = sharp).  Only a
     * reference built with DIFFUSE_REFLECTIONS uses them (ray::reflect
     * ray.cc:137-182, ray::refract ray.cc:236-280), here
     * rt_render_distributed with diffuse_samples > 0; every other render
     * ignores them, as the default build does. */
    float rfd, td;
} rt_material;
#define RT_MAT_NO_VERTEX_COLOUR 1u
#define RT_MAX_MATERIALS 16

/* Triangle flag bits (triangle.h:40, bvh_node.h:176): shadow and AO rays
 * ignore light and transparent triangles. */
#define RT_TRI_LIGHT 1u
#define RT_TRI_TRANSPARENT 2u

/* Frame statistics filled by the render calls (nullable). */
typedef struct rt_render_stats {
    int64_t primary_rays;
    int64_t secondary_rays;    /* shadow + AO rays traced */
    int64_t primary_hits;
    float device_ms;           /* device time of the render kernel(s) */
    int32_t status;            /* device status word (0 = clean) */
    int64_t nodes_fetched;     /* wide nodes loaded (RT_OPT_COUNT_FETCHES only) */
    int64_t tris_tested;       /* triangles tested (RT_OPT_COUNT_FETCHES only) */
} rt_render_stats;

/* ------------------------------------------------------------ context */

/* Create a context on CUDA device `device` (replaces nothing: the reference
 * has no device state).  The context creates its own non-blocking stream. */
rt_status rt_ctx_create(int32_t device, rt_context **out);
rt_status rt_ctx_destroy(rt_context *ctx);
/* Run all further work of this context on `stream` (a cudaStream_t); NULL
 * restores the context's own stream. */
rt_status rt_ctx_set_stream(rt_context *ctx, void *stream);
/* Wait for all work queued on the context's stream. */
rt_status rt_ctx_synchronize(rt_context *ctx);
/* Context options.  RT_OPT_COUNT_FETCHES (0/1): render calls use an
 * instrumented kernel that counts node loads and triangle tests into
 * rt_render_stats (for roofline accounting; slower, off by default). */
#define RT_OPT_COUNT_FETCHES 1
/* RT_OPT_RENDER_KERNEL: RT_KERNEL_PIXEL (default) -- one pixel per lane, a
 * warp takes the next tile when all its pixels are done; RT_KERNEL_WAVE --
 * lanes replace finished rays (primary -> secondary rays -> next pixel),
 * shading and refills batched across lanes.  Same results. */
#define RT_OPT_RENDER_KERNEL 2
#define RT_KERNEL_WAVE 0
#define RT_KERNEL_PIXEL 1
/* RT_OPT_INTERSECTOR: RT_ISECT_REFERENCE (default) -- the reference's
 * Moller-Trumbore arithmetic (triangle.h:190-235), bit-identical hits;
 * RT_ISECT_WATERTIGHT -- the watertight test of Woop, Benthin and Wald
 * (JCGT 2013): no ray passes between two triangles that share an edge; t
 * agrees with the reference to ~1e-6 relative, ids away from edges. */
#define RT_OPT_INTERSECTOR 3
#define RT_ISECT_REFERENCE 0
#define RT_ISECT_WATERTIGHT 1
/* RT_OPT_BUILDER: the binary tree that rt_bvh_build / rt_bvh_build_batched
 * collapse into 8-wide nodes.  RT_BUILDER_HPLOC (default) -- clustering of
 * mutual nearest neighbours (surface area of the merged box) run bottom-up
 * inside the Morton radix tree in one launch (H-PLOC, Benthin et al. 2024;
 * batched builds use RT_BUILDER_PLOC for it); RT_BUILDER_PLOC -- the same
 * clustering by global iterations over the Morton order (Meister and
 * Bittner 2018); RT_BUILDER_LBVH -- the Morton radix tree itself (Karras
 * 2012): fastest to build, ~10 % more nodes per ray.  Hits do not depend on
 * the tree. */
#define RT_OPT_BUILDER 4
#define RT_BUILDER_LBVH 0
#define RT_BUILDER_PLOC 1
#define RT_BUILDER_HPLOC 2
/* RT_OPT_MORTON_BITS: bits per axis of the Morton codes the builders sort
 * (10..21), or 0 (default): 21 below a million triangles, else sized from
 * the triangle count, about 3 more than log2(n) / 3, so that each Morton
 * cell holds a few triangles at most.  The radix sort orders only the bits
 * in use.  Hits do not depend on it. */
#define RT_OPT_MORTON_BITS 5
rt_status rt_ctx_set_option(rt_context *ctx, int32_t option, int64_t value);
/* Message of the last error on the calling thread ("" if none). */
const char *rt_last_error_string(void);
/* Library version as major*10000 + minor*100 + patch. */
int32_t rt_version(void);

/* -------------------------------------------------------------- scene */

/* Create an empty scene in a context. */
rt_status rt_scene_create(rt_context *ctx, rt_scene **out);
rt_status rt_scene_destroy(rt_scene *scene);

/* Upload an indexed triangle mesh.  Replaces building a primitive_store with
 * primitive_store::emplace_back(material, a, b, c, light, v_n, v_t)
 * (raytracer/primitive_store.h:29-34, triangle.h:124-176): verts_xyz holds 3
 * floats per vertex, tri_idx 3 vertex indices per triangle (a, b, c; the
 * face normal is (b-a) x (c-a)), vert_attr (nullable) 3 floats per vertex
 * (the per-vertex texture attribute, a colour in 0..1), tri_flags (nullable)
 * RT_TRI_* bits per triangle.  Invalidates any built hierarchy. */
rt_status rt_scene_upload(rt_scene *scene, const float *verts_xyz, int32_t nverts, const int32_t *tri_idx,
                          int32_t ntris, const float *vert_attr, const uint32_t *tri_flags);

/* Update vertex positions (same topology) and rebuild the hierarchy; the
 * per-frame rebuild the physics engine's render loop needs
 * (physics_engine/simulation_environment.cc:56-58). */
rt_status rt_scene_update_vertices(rt_scene *scene, const float *verts_xyz, int32_t nverts);

/* Update vertex positions (same topology) and refit the existing hierarchy
 * instead of rebuilding it: shading records and boxes recomputed bottom-up,
 * every wide node re-quantised, the tree's topology kept.  The cheap
 * per-frame path for small motions of the same physics-engine loop
 * (physics_engine/simulation_environment.cc:56-58); hits are exact as after
 * a rebuild, traversal slows as the motion departs from the built layout.
 * Requires a built scene.  refit_ms (nullable): device time. */
rt_status rt_scene_refit_vertices(rt_scene *scene, const float *verts_xyz, int32_t nverts, float *refit_ms);

/* Build the acceleration structure: GPU Morton LBVH collapsed to 8-wide
 * nodes with 8-bit conservatively quantised child boxes.  Replaces
 * bvh::bvh(primitive_store&) -> bvh_builder::build
 * (spatial_sub_division/bvh.h:27-32, bvh_builder.cc:18-178).  build_ms
 * (nullable) receives the device build time. */
rt_status rt_bvh_build(rt_scene *scene, float *build_ms);

/* Hierarchy statistics: wide nodes, packed triangle slots, tree depth. */
rt_status rt_bvh_info(const rt_scene *scene, int32_t *nodes, int32_t *tri_slots, int32_t *depth);

/* Child-slot usage of the built hierarchy (copies the nodes to the host). */
typedef struct rt_bvh_stats {
    int64_t nodes;
    int64_t internal_slots;    /* child slots holding an internal node */
    int64_t leaf_slots;        /* child slots holding 1..3 triangles */
    int64_t empty_slots;
    int64_t leaf_tris[4];      /* leaf slots by triangle count (index 1..3) */
} rt_bvh_stats;
rt_status rt_bvh_stats_get(const rt_scene *scene, rt_bvh_stats *out);

/* ---------------------------------------------------------- traversal */

/* Closest hit for n rays.  Replaces ssd::find_nearest_object(const ray*,
 * hit_description*) (spatial_sub_division/ssd.h:26-44) as implemented by
 * bvh::find_nearest_object (bvh.cc:649-709).  Accepts t > 1e-3 (EPSILON);
 * among equal t the lowest triangle id wins. */
rt_status rt_trace_closest(rt_scene *scene, const rt_ray *rays, int32_t n, rt_hit *hits);

/* Any hit with 1e-3 < t < ray.tmax for n rays, skipping light and
 * transparent triangles.  Replaces ssd::found_nearer_object(const ray*,
 * float t) (ssd.h, bvh.cc:711-759, bvh_node.h:170-190).  occluded[i] is 1
 * when ray i is blocked. */
rt_status rt_trace_any(rt_scene *scene, const rt_ray *rays, int32_t n, uint8_t *occluded);

/* Closest hit, as rt_trace_closest, for callers that cannot allocate device
 * memory (an engine whose allocator owns the whole GPU, a real-time loop
 * that forbids allocation after start-up).  No counterpart in the
 * reference.  Calls no cudaMalloc or cudaFree: rays and hits (host or
 * device memory) are staged through one fixed scratch array of
 * RT_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit.  At most RT_NOALLOC_MAX_RAYS rays per call (RT_ERR_INVALID_ARG
 * beyond).  The first call on a device looks up the array's address; make
 * it before any stream capture.  All calls share the array: calls that
 * overlap on the GPU race, so serialise them (each call synchronises the
 * context's stream before it returns). */
#define RT_NOALLOC_MAX_RAYS 16384
#define RT_NOALLOC_SCRATCH_BYTES (256 + RT_NOALLOC_MAX_RAYS * 48)
rt_status rt_trace_closest_noalloc(rt_scene *scene, const rt_ray *rays, int32_t n, rt_hit *hits);

/* ------------------------------------------------------------- render */

/* Render one frame: primary ray per pixel, closest hit, one shadow ray per
 * light from the offset hit point, coloured Phong, clamp-and-truncate to
 * RGB8, all in one fused kernel.  Replaces ray_tracer(const ssd*, const
 * light_list&, const primitive_store&, camera&) (raytracer.h:105,
 * raytracer.cc:563-598) followed by camera::clip_image_to_rgb
 * (camera.h:289-319).  rgb_out: xres*yres*3 bytes, row 0 at the bottom.
 * hit_ids (nullable): primary-hit triangle id per pixel (-1 = background).
 * Up to RT_MAX_LIGHTS lights. */
#define RT_MAX_LIGHTS 8
rt_status rt_render(rt_scene *scene, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                    const rt_material *material, uint8_t *rgb_out, int32_t *hit_ids, rt_render_stats *stats);

/* Per-triangle materials: mat_of_tri[i] (ntris entries, host or device
 * memory) indexes the table given to rt_render_materials; NULL returns every
 * triangle to material 0.  The reference keeps a material pointer per
 * triangle (triangle.h:99-106). */
rt_status rt_scene_set_materials(rt_scene *scene, const int32_t *mat_of_tri, int32_t ntris);

/* Per-triangle corner normals for smooth shading: 9 floats per triangle
 * (normals at vertices a, b, c; host or device memory), interpolated by
 * the hit's barycentrics into the shading normal as the reference's
 * triangle::normal_at_point does with vertex normals (triangle.h:473-476);
 * a triangle whose first float is FLT_MAX keeps its face normal.  NULL
 * removes them.  Shadow and secondary ray origins keep the face normal. */
rt_status rt_scene_set_normals(rt_scene *scene, const float *corner_normals, int32_t ntris);

/* rt_render with a table of up to RT_MAX_MATERIALS materials indexed per
 * triangle: every hit is shaded with its triangle's material, and mirror
 * (rf) and refracted (tran, ri) rays are traced as a tree, reflection
 * before refraction, each colour added times its weight
 * (ray_trace_engine::ray_trace, raytracer.cc:20-87, and
 * combind_secondary_rays, coloured_mapper_shader.cc:117-130).  At most
 * RT_MAX_BOUNCES levels and RT_MAX_TREE_RAYS rays per pixel (tables needing
 * more are refused).  Without rt_scene_set_materials every triangle takes
 * materials[0]; rt_render is the one-material case and ignores the
 * per-triangle indices.  Every index set on the scene must be below
 * nmaterials. */
/* The camera's float image: what ray_tracer() (raytracer.cc:563-598)
 * stores through camera::set_pixel (camera.h:281-285) before
 * clip_image_to_rgb or tone_map read it -- the unclipped colour of every
 * ray of the camera grid given (pass the supersampled grid, xres * x_a_res
 * by yres * y_a_res, for an anti-aliased camera), 3 floats per sample,
 * index x + y * xres.  Materials as rt_render_materials (one entry, or a
 * table indexed per triangle; mirror and refracting materials trace their
 * ray trees), the specular power evaluated exactly.  rgb_f32 is host or
 * device memory. */
rt_status rt_render_image(rt_scene *scene, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                          const rt_material *materials, int32_t nmaterials, float *rgb_f32, rt_render_stats *stats);

rt_status rt_render_materials(rt_scene *scene, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                              const rt_material *materials, int32_t nmaterials, uint8_t *rgb_out, int32_t *hit_ids,
                              rt_render_stats *stats);

/* ------------------------------------------------------- scene ingest */

/* A triangle mesh read from a file, triangulated as the reference's parsers
 * triangulate it and in the order they fill its primitive_store, so triangle
 * i here is primitive i there (raytracer/parsers/off_parser.cc:15-100,
 * ply_parser.cc:480-583, obj_parser.cc:762-857, polygon_to_triangles.h:
 * 240-389).  verts: 3 floats per vertex; tris: 3 vertex indices per triangle
 * (rt_scene_upload's arrays); tri_rgb: 3 bytes per triangle when the file
 * colours its faces (binary PLY), else NULL; tri_mat: per triangle the
 * material of an OBJ file (0: the default, i: the i-th distinct usemtl name
 * in order of first use; nmat of them), else NULL; kd: the parser's default
 * diffuse colour (OFF 170, PLY and OBJ 200).  OBJ vertex normals come
 * back per triangle corner (normalised, as parse_vn_statement does); OBJ
 * material libraries (mtllib) and texture coordinates are read past, not
 * returned.  Arrays are malloc'd; rt_mesh_free releases them. */
#define RT_MESH_AUTO 0   /* by file extension: .off, .ply, .obj */
#define RT_MESH_OFF 1
#define RT_MESH_PLY 2    /* format ascii 1.0 or binary_big_endian 1.0 */
#define RT_MESH_OBJ 3
typedef struct rt_mesh {
    int32_t nverts, ntris;
    float *verts;
    int32_t *tris;
    uint8_t *tri_rgb;
    float kd[3];
    int32_t *tri_mat;
    int32_t nmat;
    float *corner_normals;   /* OBJ vertex normals: 9 floats per triangle for rt_scene_set_normals
                                (FLT_MAX first: none), or NULL */
} rt_mesh;
rt_status rt_mesh_load(const char *path, int32_t format, rt_mesh *out);
rt_status rt_mesh_parse(const char *data, int64_t len, int32_t format, rt_mesh *out);
void rt_mesh_free(rt_mesh *mesh);

/* Framebuffer epilogue: the reference's global and histogram tone mapping
 * (camera::tone_map, raytracer/camera.cc:1124-1463, with glare and temporal
 * adaptation off; mode values of tone_mapping_mode_t, camera.h:43-45) and
 * gamma correction (camera::gamma_correct, camera.cc:1466-1500).  key, xw,
 * yw, desaturate and stretch are tone_map's key, xw, yw, ds and sc (its
 * defaults: 0.18, 1/3, 1/3, 0, 0); gamma > 0 applies gamma_correct(gamma)
 * after tone mapping (2.2 selects the sRGB curve, as in the reference), 0
 * none.  The histogram modes (camera::histogram_tone_map, camera.cc:
 * 1843-2062) resample the frame to one block per degree of the camera's
 * view and need a view of 2 to 4096 degrees each way (measured as the
 * reference measures it: 2w/t and 2h/t radians).  The bilateral mode
 * (camera::bilateral_filter_tone_map(0.4, s, 0.4, s), s = 0.02 * min(w,
 * h), camera.cc:1354-1358, 1632-1812) runs the reference's bilateral grid
 * with its Gaussian blur computed exactly (the reference's FFTW rounding
 * is not reproduced, so a pixel may differ by a level); like the reference
 * it compresses the base to a contrast of 300 without removing its
 * maximum, so frames of ordinary brightness saturate.  A sample at or below
 * the 3.18e-7 luminance floor, which the reference leaves unset, counts as
 * log-luminance 0.  Frames whose grid would exceed 2^26 cells (extreme
 * aspect ratios) are refused. */
#define RT_TONE_NONE 0
#define RT_TONE_GLOBAL_CONTRAST 1
#define RT_TONE_LOCAL_HISTOGRAM 2          /* camera::histogram_tone_map(false) */
#define RT_TONE_LOCAL_HUMAN_HISTOGRAM 3    /* histogram_tone_map(true): visibility-limited */
#define RT_TONE_GLOBAL_NON_LINEAR 4
#define RT_TONE_GLOBAL_EXPOSURE 5
#define RT_TONE_GLOBAL_AVG_LUMINANCE 6
#define RT_TONE_GLOBAL_MAX_LUMINANCE 7
#define RT_TONE_GLOBAL_BILATERAL 8
#define RT_TONE_GLOBAL_FERWERDA 9
typedef struct rt_tone_map {
    int32_t mode;
    float key, xw, yw;
    int32_t desaturate, stretch;
    float gamma;
} rt_tone_map;

/* A frame of rt_render_materials traced on the anti-aliased grid (aa_x *
 * aa_y rays per output pixel, 1..16 each), kept as floats, tone mapped and
 * gamma corrected as a whole (tone NULL: neither), then averaged per output
 * pixel, clamped and truncated to RGB8 (camera::clip_image_to_rgb,
 * camera.h:289-319).  Replaces ray_tracer + camera::tone_map +
 * camera::gamma_correct + clip_image_to_rgb.  The luminance statistics of
 * the tone mappers are summed in double where the reference sums binary32
 * in pixel order, so frames may differ from the reference's by one level in
 * a few pixels. */
rt_status rt_render_tone_mapped(rt_scene *scene, const rt_camera *camera, int32_t aa_x, int32_t aa_y,
                                const rt_light *lights, int32_t nlights, const rt_material *materials,
                                int32_t nmaterials, const rt_tone_map *tone, uint8_t *rgb_out,
                                rt_render_stats *stats);

/* The tone map of rt_render_tone_mapped applied to a given float frame
 * (3 floats per sample in 0..255 units, the camera's xres * aa_x by
 * yres * aa_y grid, row 0 at the bottom; host or device), e.g. one made by
 * rt_render_float: camera::tone_map + gamma_correct + clip_image_to_rgb on
 * a camera whose image is that frame. */
rt_status rt_tone_map_image(rt_context *ctx, const rt_camera *camera, int32_t aa_x, int32_t aa_y, const float *fimg,
                            const rt_tone_map *tone, uint8_t *rgb_out);

/* Diagnostic of the tone mapper's log10 (float-float evaluation, rounded
 * once): on n positive floats drawn from every binade (seeded), counts the
 * values whose decided result differs from log10 evaluated in double and
 * rounded (*mismatches, expected 0) and the values left to the double
 * evaluation (*undecided). */
rt_status rt_check_log10(rt_context *ctx, int64_t n, uint64_t seed, int64_t *mismatches, int64_t *undecided);

/* The binary32 sum of values[0..n) in index order, rounded after every
 * addition exactly as a sequential loop `s += values[i]` rounds it (the way
 * camera::tone_map accumulates its log-luminance, camera.cc:1158), computed
 * on the GPU; rt_render_tone_mapped uses the same machinery.  values: host
 * or device, finite. */
rt_status rt_sum_sequential_f32(rt_context *ctx, const float *values, int64_t n, float *sum_out);

/* Anti-aliased frame: aa_x * aa_y rays per output pixel on the supersampled
 * camera grid (xres * aa_x by yres * aa_y), each shaded as by rt_render, and
 * their colours averaged into the xres * yres RGB8 output.  Replaces the
 * reference camera built with anti-aliasing factors x_a_res / y_a_res
 * (raytracer/camera.h:55-62) rendered by ray_tracer and downsampled by
 * camera::clip_image_to_rgb (camera.h:289-319: samples summed x outer, y
 * inner, divided by their count, clamped, truncated).  aa_x, aa_y in 1..16. */
rt_status rt_render_aa(rt_scene *scene, const rt_camera *camera, int32_t aa_x, int32_t aa_y, const rt_light *lights,
                       int32_t nlights, const rt_material *material, uint8_t *rgb_out, rt_render_stats *stats);

/* Ambient-occlusion render (no reference counterpart; the reference has no
 * AO): primary closest hit, then `samples` cosine-weighted hemisphere rays
 * per hit (Philox4x32-10 keyed by pixel and sample, seed) from the offset hit
 * point, any-hit within `ao_dist`.  Pixel = ka + kd * unoccluded fraction.
 * ao_count (nullable): unoccluded rays per pixel.  samples <= 64. */
rt_status rt_render_ao(rt_scene *scene, const rt_camera *camera, const rt_material *material, int32_t samples,
                       float ao_dist, uint32_t seed, uint8_t *rgb_out, int32_t *hit_ids, int32_t *ao_count,
                       rt_render_stats *stats);

/* ------------------------------------------------------ soft shadows */

#define RT_MAX_SOFT_SAMPLES 64

/* The extent of a light for rt_render_soft_shadows, one per light:
 * radius is the radius r of a spherical light (the reference's spherical
 * and spot-light constructors, light.h:17-18, 24-25); a light with
 * ntris > 0 is instead defined by triangles of the scene (its triangle
 * constructors, light.h:20-21, 27-29): tris lists ntris indices into the
 * scene's triangles (the caller's order; host memory borrowed for the
 * call), which should carry RT_TRI_LIGHT so shadow rays pass them, radius
 * is then 0, and the light's pos is its centre. */
typedef struct rt_light_shape {
    float radius;
    int32_t ntris;
    const int32_t *tris;
} rt_light_shape;

/* Soft shadows as RAPTor renders them when it is built with SOFT_SHADOW =
 * samples (ray::find_rays ray.cc:91-104, light::find_rays light.h:62-164,
 * ray_trace_engine::ray_trace raytracer.cc:44-64): every primary hit sends
 * `samples` shadow rays to random points of each spherical or
 * triangle-defined light (RT_LIGHT_POINT and RT_LIGHT_SPOT; shapes[l] as
 * above, NULL: all spherical with radius 0) and one ray to each directional
 * light; a light's term is shaded with its first ray's direction and length
 * and weighted by the fraction of its rays that reach it.  The random
 * points are the reference's own: its process-wide generator
 * (common/common.cc:35-105) draws, in pixel order (x + y * xres) and light
 * order, three numbers per ray of a spherical light and two per ray a
 * triangle-defined light makes (triangle::find_rays, triangle.h:504-525;
 * samples / ntris rays per triangle plus one for the triangles its stride
 * lands on, light.h:131-156, which is samples + 1 rays when ntris divides
 * samples -- the reference's release build draws for all of them and
 * traces the first `samples`; a light making fewer is refused).
 * stream_offset says how many numbers the generator had produced before
 * this frame (0: a freshly started program); stream_end (nullable)
 * receives the count after the frame, the next frame's offset.  Frames
 * without mirror or refracting materials (`materials` as
 * rt_render_materials).  rgb_out (RGB8) and rgb_f32 (the camera's float
 * image) are nullable, not both, host or device memory.  Runs two passes
 * with one host round trip between them: the camera rays, then the frame's
 * slice of the random stream (generated on the host and copied over unless
 * the previous frame's slice already covers it) and the shading. */
rt_status rt_render_soft_shadows(rt_scene *scene, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                                 const rt_light_shape *shapes, const rt_material *materials, int32_t nmaterials,
                                 int32_t samples, int64_t stream_offset, uint8_t *rgb_out, float *rgb_f32,
                                 int64_t *stream_end, rt_render_stats *stats);

/* -------------------------------------------- distributed ray tracing */

#define RT_STREAM_REFERENCE 0
#define RT_STREAM_PIXEL 1

/* What a distributed frame samples and where its random numbers come from.
 * soft_samples: SOFT_SHADOW, 1..RT_MAX_SOFT_SAMPLES (1: the default build);
 * diffuse_samples: DIFFUSE_REFLECTIONS, 0..RT_MAX_SOFT_SAMPLES (0: the
 * default build).  stream: RT_STREAM_REFERENCE draws the reference's own
 * process-wide generator (common/common.cc:35-105) in the reference's
 * order, pixel after pixel from position stream_offset; RT_STREAM_PIXEL
 * gives every node of every pixel's ray tree its own stream -- number k
 * that node q of pixel p draws is word k % 4 of Philox4x32-10 (Salmon et
 * al., SC'11) with counter (p, q low, q high, k / 4) and key (seed low,
 * seed high), as (float)word * 2^-32, the reference generator's conversion;
 * the camera ray is node 0x6A09E667F3BCC909 and ray i of a node's
 * reflection (s = 0) or refraction (s = 1) set is node SplitMix64(q + (64 s
 * + i + 1) * 0x9E3779B97F4A7C15) -- drawn in the reference's order within
 * the node (the lights' rays, then the reflection set, then the refraction
 * set).  Keyed by node, a subtree's numbers do not depend on how many its
 * elder siblings drew, so the subtrees of a pixel are traced in parallel. */
typedef struct rt_sampling {
    int32_t soft_samples;
    int32_t diffuse_samples;
    int32_t stream;
    int32_t reserved;          /* 0 */
    int64_t stream_offset;     /* RT_STREAM_REFERENCE */
    uint64_t seed;             /* RT_STREAM_PIXEL */
} rt_sampling;

/* Distributed ray tracing as RAPTor renders a frame when it is built with
 * SOFT_SHADOW = soft_samples and DIFFUSE_REFLECTIONS = diffuse_samples
 * (ray_trace_engine::ray_trace raytracer.cc:20-87, ray::find_rays
 * ray.cc:91-104, ray::reflect ray.cc:118-182, ray::refract ray.cc:198-281,
 * light::find_rays light.h:62-164, combind_secondary_rays
 * coloured_mapper_shader.cc:117-130).  Every ray carries a componant c
 * (1 for camera rays); at each hit, max(soft_samples / c, 1) shadow rays go
 * to each spherical or triangle-defined light (shapes as for
 * rt_render_soft_shadows) and one to each directional light; a reflection
 * of power magn * rf above 0.1 is one mirror ray, or -- with
 * diffuse_samples > 0 and the material's rfd != 0 -- max(diffuse_samples /
 * c, 1) rays spread about the mirror direction by rfd, each of componant
 * 4c; refractions likewise with tran, ri and td; each set's mean colour is
 * added times rf, then tran.  Limits of rt_render_materials on the tree.
 * RT_STREAM_REFERENCE renders the reference's frame exactly (one counting
 * pass over the ray trees fixes every pixel's position in the stream; the
 * frame's slice is generated on the host), but not with diffuse rays,
 * whose count depends on where earlier random rays of the frame landed:
 * replaying one stream through them is serial, so such frames need
 * RT_STREAM_PIXEL.  stream_end (nullable) receives, for
 * RT_STREAM_REFERENCE, the generator's position after the frame; for
 * RT_STREAM_PIXEL, the numbers the frame drew.  rgb_out / rgb_f32 as for
 * rt_render_soft_shadows. */
rt_status rt_render_distributed(rt_scene *scene, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                                const rt_light_shape *shapes, const rt_material *materials, int32_t nmaterials,
                                const rt_sampling *sampling, uint8_t *rgb_out, float *rgb_f32, int64_t *stream_end,
                                rt_render_stats *stats);

/* ---------------------------------------------------- differentiation */

/* Replace the per-vertex attributes (colours) without touching geometry. */
rt_status rt_scene_update_attributes(rt_scene *scene, const float *vert_attr, int32_t nverts);

/* rt_render's frame as unclipped float colours (the camera's ext_colour_t
 * image before camera::clip_image_to_rgb, camera.h:281-319): rgb_f32
 * xres*yres*3 floats, hit_ids (nullable) the primary hit per pixel,
 * occluded (nullable) per pixel a bit per light set when its shadow ray was
 * blocked.  All outputs DEVICE memory. */
rt_status rt_render_float(rt_scene *scene, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                          const rt_material *material, float *rgb_f32, int32_t *hit_ids, uint8_t *occluded,
                          rt_render_stats *stats);

/* Adjoint of rt_render_float (no reference counterpart): given dL/dpixel
 * (xres*yres*3 floats), writes dL/dvertex-position and dL/dvertex-attribute
 * (nverts*3 floats each, zeroed first).  Interior gradients: the hit
 * triangle and shadow-ray visibility of every pixel are held fixed.  The
 * kernel re-traces each pixel instead of storing hit records (memory
 * O(pixels + vertices)).  All buffers DEVICE memory. */
rt_status rt_render_adjoint(rt_scene *scene, const rt_camera *camera, const rt_light *lights, int32_t nlights,
                            const rt_material *material, const float *dL_dpix, float *dL_dpos, float *dL_dattr,
                            rt_render_stats *stats);

/* ------------------------------------------------------------ batches */

/* A batch renders many scenes (own hierarchy, resolution and ray mix each)
 * in ONE persistent launch fed by a device work queue of 32-pixel tiles,
 * replayed from a captured CUDA graph.  No reference counterpart: the
 * reference renders one scene per ray_tracer() call (raytracer.cc:563). */
typedef struct rt_batch rt_batch;

#define RT_JOB_SHADOW 0        /* primary + one shadow ray per light, Phong */
#define RT_JOB_AO 1            /* primary + ao_samples AO rays, AO shading */
#define RT_MAX_JOB_LIGHTS 2
typedef struct rt_job {
    int32_t scene;             /* index from rt_batch_add_scene */
    int32_t mode;              /* RT_JOB_SHADOW or RT_JOB_AO */
    rt_camera camera;
    int32_t nlights;           /* RT_JOB_SHADOW: 0..RT_MAX_JOB_LIGHTS */
    rt_light lights[RT_MAX_JOB_LIGHTS];
    rt_material material;
    int32_t ao_samples;        /* RT_JOB_AO: 1..64 */
    float ao_dist;
    uint32_t ao_seed;
    uint8_t *rgb_out;          /* DEVICE memory, xres*yres*3 */
    int32_t *hit_ids;          /* DEVICE memory or NULL */
} rt_job;

/* Launch shape of the batched kernel, chosen by rt_batch_autotune:
 * threads per block (64/128/256), tiles claimed per queue access (1..16,
 * RT_KERNEL_PIXEL only: the queue depth a warp takes at once), tile width
 * (8 -> 8x4 tiles, 16 -> 16x2), kernel (RT_KERNEL_WAVE / RT_KERNEL_PIXEL,
 * see RT_OPT_RENDER_KERNEL), the measured ms per frame, and the traversal
 * stack capacity in node groups (16, 24 or 48, RT_KERNEL_PIXEL only; at
 * least the depth of the batch's deepest tree). */
typedef struct rt_tune_config {
    int32_t block_threads;
    int32_t chunk_tiles;
    int32_t tile_w;
    int32_t kernel;
    float ms;
    int32_t stack_entries;
} rt_tune_config;

rt_status rt_batch_create(rt_context *ctx, rt_batch **out);
rt_status rt_batch_destroy(rt_batch *batch);
/* Add a scene (same arguments as rt_scene_upload); scene_index receives its
 * index.  Up to 1024 scenes, 2^28 triangles in total. */
rt_status rt_batch_add_scene(rt_batch *batch, const float *verts_xyz, int32_t nverts, const int32_t *tri_idx,
                             int32_t ntris, const float *vert_attr, const uint32_t *tri_flags, int32_t *scene_index);
/* Build every scene's hierarchy in one batched LBVH pass. */
rt_status rt_bvh_build_batched(rt_batch *batch, float *build_ms);
/* Set the frames to render (re-captures the graph). */
rt_status rt_batch_set_jobs(rt_batch *batch, const rt_job *jobs, int32_t njobs);
/* Render all jobs: one graph launch on the context's stream.  With stats ==
 * NULL the call returns without waiting; otherwise it waits and fills
 * stats (device_ms = graph time). */
rt_status rt_render_batched(rt_batch *batch, rt_render_stats *stats);
/* Time every launch shape on the current jobs (reps graph replays each) and
 * keep the fastest; best (nullable) receives it. */
rt_status rt_batch_autotune(rt_batch *batch, int32_t reps, rt_tune_config *best);
rt_status rt_batch_set_config(rt_batch *batch, const rt_tune_config *config);
rt_status rt_batch_get_config(const rt_batch *batch, rt_tune_config *config);

#ifdef __cplusplus
}
#endif
#endif
