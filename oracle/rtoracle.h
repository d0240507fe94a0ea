/*
 * rtoracle.h -- CPU restatement of RAPTor's ray-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the CUDA core is
 * compared against: tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it; the product library never does.
 *
 * Every function restates the reference's scalar CPU path (file:line given
 * beside each declaration, paths relative to the RAPTor project root).  All
 * arithmetic is IEEE binary32 in the reference's operation order; the library
 * is compiled with -ffp-contract=off so x86 and Arm give identical bits.
 *
 * The one deliberate difference from the reference: the hierarchy above the
 * Morton-sorted primitives is a top-down split on the highest differing Morton
 * bit instead of the reference's approximate agglomerative clustering
 * (raytracer/spatial_sub_division/bvh_builder.cc:292-642).  The traversal
 * (bvh.cc:586-759) returns the closest accepted intersection whatever the tree
 * shape, so hits differ only where two triangles give bit-identical distances
 * (the reference keeps the first one found).  The tests pin this restatement
 * hit-for-hit against the reference itself where it can be compiled.
 */
#ifndef RTORACLE_H
#define RTORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Camera as the reference's camera constructor takes it
 * (raytracer/camera.h:55-62): position, x/y/z axes, background colour,
 * half-width w, half-height h, image-plane distance t, resolution. */
typedef struct ro_camera {
    float pos[3];
    float x_axis[3], y_axis[3], z_axis[3];
    float background[3];
    float w, h, t;
    int32_t xres, yres;
} ro_camera;

/* Light (raytracer/light.h:17-34).  kind 0 = point light at pos (the
 * spherical-light constructor with soft shadows off), kind 1 = directional
 * light along dir.  rgb is in 0..255 units, d is the distance drop-off. */
typedef struct ro_light {
    int32_t kind;
    float rgb[3];
    float pos[3];
    float dir[3];
    float d;
    float s_a, s_b;   /* kind 2 (spot light at pos, axis dir): cone angles, light.h:24-25 */
    float r;          /* kinds 0 and 2: radius of the spherical light (light.h:17-25); used by soft shadows */
    int32_t ntris;    /* kinds 0 and 2: a triangle-defined light (light.h:20-21, 27-29) -- its ntris */
    const int32_t *tris;  /* triangles (scene indices, flagged RO_TRI_LIGHT); pos is its centre.  NULL / 0: none */
} ro_light;

/* Coloured-mapper Phong material (materials/coloured_mapper_shader.h): ka,
 * kd, ks in 0..255 units, ns the specular exponent.  When the scene carries
 * per-vertex attributes, kd is modulated by the interpolated attribute
 * (attribute * 255 sampled, then scaled by kd / 255). */
typedef struct ro_material {
    float ka[3], kd[3], ks[3];
    float ns;
    float rf;     /* mirror reflectivity, coloured_mapper_shader's rf (0: none) */
    float tran;   /* transparency: refracted colour weight, the shader's tran (0: none) */
    float ri;     /* refractive index, the shader's ri */
    uint32_t flags;   /* RO_MAT_NO_VERTEX_COLOUR: kd not modulated by the vertex attribute */
    float rfd;    /* spread of a diffuse reflection, the shader's rfd (0: sharp); DIFFUSE_REFLECTIONS builds only */
    float td;     /* spread of a diffuse refraction, the shader's td (0: sharp); DIFFUSE_REFLECTIONS builds only */
} ro_material;
#define RO_MAT_NO_VERTEX_COLOUR 1u

typedef struct ro_scene ro_scene;

/* Triangle-flag bits: bit 0 marks a light (ignored by shadow rays,
 * triangle.h:40), bit 1 a transparent material (bvh_node.h:176). */
#define RO_TRI_LIGHT       1u
#define RO_TRI_TRANSPARENT 2u

/* Morton code of a point (common/simd.h:798-825), truncating float->int. */
int32_t ro_morton_code(float x, float y, float z, float x_mul, float y_mul, float z_mul);

/* Scene from an indexed mesh; vattr (3 floats per vertex) and flags may be
 * NULL.  Triangle i keeps id i, as primitive_store::indirection does. */
ro_scene *ro_scene_create(const float *verts, int32_t nverts, const int32_t *tris, int32_t ntris,
                          const float *vattr, const uint32_t *flags);
void ro_scene_destroy(ro_scene *s);

/* Build the 2-wide BVH (Morton + stable LSD radix as bvh_builder.cc:18-158).
 * Returns build seconds, or a negative value on failure. */
double ro_scene_build(ro_scene *s);
int32_t ro_scene_node_count(const ro_scene *s);

/* Closest hit for n rays (bvh.cc:649-709 + triangle.h:190-235).  ogn and dir
 * hold 3 floats per ray; id is -1 on a miss, t is FLT_MAX on a miss. */
int32_t ro_trace_closest(const ro_scene *s, const float *ogn, const float *dir, int32_t n,
                         int32_t *id, float *t, float *u, float *v);

/* Any hit strictly inside (EPSILON, tmax) for n rays (bvh.cc:711-759,
 * bvh_node.h:170-190). */
int32_t ro_trace_any(const ro_scene *s, const float *ogn, const float *dir, const float *tmax,
                     int32_t n, uint8_t *occluded);

/* Primary rays of a pixel window (camera.h:127-140): origin = camera position,
 * direction normalised with sqrt + divide (EXACT_NORMALISE). */
void ro_camera_rays(const ro_camera *cam, int32_t x0, int32_t y0, int32_t w, int32_t h,
                    float *ogn, float *dir);

/* Render rows [row0, row1) of the frame with nthreads threads
 * (raytracer.cc:20-87 per pixel, then camera.h:289-319 to RGB8).
 * rgb holds 3 bytes per pixel of the full frame, row y=0 at the bottom as in
 * the reference; hit_id (nullable) receives the primary hit id per pixel,
 * occl (nullable) the shadow-ray result per pixel and light (1 = occluded),
 * fimg (nullable) the unclipped float colour.  Returns rays traced. */
int64_t ro_render(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                  const ro_material *mat, int32_t row0, int32_t row1, int32_t nthreads,
                  uint8_t *rgb, int32_t *hit_id, uint8_t *occl, float *fimg);

/* Per-triangle corner normals (9 floats per triangle, NULL: none; a
 * triangle whose first float is FLT_MAX keeps its face normal): the shading
 * normal interpolates them as triangle::normal_at_point does with vertex
 * normals (triangle.h:464-498). */
int32_t ro_scene_set_normals(ro_scene *s, const float *corner_normals);

/* Per-triangle materials: mat_of_tri[i] indexes the table given to
 * ro_render_mt (NULL: every triangle uses material 0). */
int32_t ro_scene_set_materials(ro_scene *s, const int32_t *mat_of_tri);

/* ro_render with a material table (the reference's per-triangle material
 * pointers, triangle.h:99-106): reflections (rf) and refractions (tran, ri)
 * are traced recursively as ray_trace_engine::ray_trace does.  Shadow rays
 * pass the triangles flagged RO_TRI_TRANSPARENT; the reference passes those
 * whose material has tran > 0 (material::is_transparent, material.h:63), so
 * the flags are to agree with the table. */
int64_t ro_render_mt(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                     const ro_material *mats, int32_t nmats, int32_t row0, int32_t row1, int32_t nthreads,
                     uint8_t *rgb, int32_t *hit_id, uint8_t *occl, float *fimg);

/* Ambient-occlusion render (no reference counterpart: the ray generator is
 * this project's, restated identically in the CUDA core).  Per primary hit,
 * nsamples cosine-weighted rays from the offset hit point, any-hit within
 * ao_dist.  Pixel = ka + kd_colour * unoccluded_fraction.  ao_count (nullable)
 * receives the unoccluded-ray count per pixel. */
int64_t ro_render_ao(const ro_scene *s, const ro_camera *cam, const ro_material *mat,
                     int32_t nsamples, float ao_dist, uint32_t seed, int32_t row0, int32_t row1,
                     int32_t nthreads, uint8_t *rgb, int32_t *hit_id, int32_t *ao_count);

/* The secondary rays the camera ray of pixel (x, y) spawns, exactly as the
 * renders above trace them: with ao_n > 0 the ao_n rays of ro_ao_rays
 * (tmax = ao_dist), else one shadow ray per light (raytracer.cc:44-64,
 * light.h:62-100; tmax = the distance to the light).  hit_id receives the
 * primary hit (-1: miss, no rays).  ogn / dir hold 3 floats per ray and tmax
 * one, room for max(ao_n, nlights) rays.  Returns the number of rays, or -1
 * on bad arguments.  Lets a test re-trace exactly the rays on which two
 * renders disagree. */
int32_t ro_pixel_secondary_rays(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                                int32_t ao_n, float ao_dist, uint32_t ao_seed, int32_t x, int32_t y,
                                int32_t *hit_id, float *ogn, float *dir, float *tmax);

/* Soft shadows as the reference renders them when built with
 * SOFT_SHADOW = samples (ray.cc:91-104, light.h:62-164, raytracer.cc:44-64):
 * every primary hit sends `samples` shadow rays to random points of each
 * spherical light (kinds 0 and 2 with a cone; radius r) -- three numbers of
 * the reference's random stream per ray, drawn in pixel order (x + y * xres)
 * and light order -- or of each triangle-defined light (ntris > 0, r = 0:
 * two numbers per ray the light makes, triangle.h:504-525), and one ray to
 * each directional light; a light's term is shaded with its first ray's
 * direction and length and weighted by the unoccluded fraction.
 * stream_offset: how many numbers the reference's generator had produced
 * before the frame; stream_end (nullable) receives the count after it.
 * Materials without reflection or refraction, light triangles in range and
 * making at least `samples` rays (-1 otherwise).  Whole frame; returns rays
 * traced. */
int64_t ro_render_soft(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                       const ro_material *mats, int32_t nmats, int32_t samples, int64_t stream_offset,
                       int32_t nthreads, uint8_t *rgb, int32_t *hit_id, float *fimg, int64_t *stream_end);

/* The rays light::find_rays makes for a triangle-defined light of ntris
 * triangles asked for n (light.h:129-164): n / ntris per triangle and one
 * more for every triangle the binary32 stride lands on.  cnt (nullable,
 * ntris entries) receives each triangle's count; returns their sum, which
 * is n + 1 when ntris divides n (the reference's assert on the sum is
 * compiled out of its release build, which draws for every ray made and
 * traces the first n), or -1 for ntris < 1 or n < 1. */
int32_t ro_area_light_rays(int32_t ntris, int32_t n, int32_t *cnt);

/* Distributed ray tracing as the reference renders it when built with
 * SOFT_SHADOW = soft and DIFFUSE_REFLECTIONS = diffuse
 * (ray_trace_engine::ray_trace raytracer.cc:20-87 with ray::find_rays
 * ray.cc:91-104, ray::reflect ray.cc:118-182, ray::refract ray.cc:198-281,
 * light::find_rays light.h:62-164 and combind_secondary_rays
 * coloured_mapper_shader.cc:117-130): at every hit of a ray of componant c
 * (1 for camera rays), max(soft / c, 1) shadow rays per spherical or
 * triangle-defined light; a reflection (power magn * rf above 0.1) is one
 * mirror ray, or with diffuse > 0 and the material's rfd != 0,
 * max(diffuse / c, 1) rays spread by rfd about it, each of componant 4c;
 * refractions the same with tran and td; each set's mean colour is added
 * times rf, then tran.  The random numbers come, in the reference's order
 * within a pixel, from stream: RO_STREAM_REFERENCE, the reference's own
 * process-wide generator from position offset, pixels in the reference's
 * order (x + y * xres) -- serial, nthreads ignored; RO_STREAM_PIXEL, one
 * stream per pixel and tree node (ro_pixel_stream with seed).  drawn (nullable) receives
 * the count of numbers the frame drew.  Returns rays traced, or -1 on bad
 * arguments. */
typedef struct ro_sampling {
    int32_t soft;       /* SOFT_SHADOW: 1..64 (1: the default build) */
    int32_t diffuse;    /* DIFFUSE_REFLECTIONS: 0..64 (0: the default build) */
    int32_t stream;     /* RO_STREAM_REFERENCE or RO_STREAM_PIXEL */
    int32_t reserved;
    int64_t offset;     /* RO_STREAM_REFERENCE: numbers drawn before the frame */
    uint64_t seed;      /* RO_STREAM_PIXEL: the streams' key */
} ro_sampling;
#define RO_STREAM_REFERENCE 0
#define RO_STREAM_PIXEL 1
int64_t ro_render_distributed(const ro_scene *s, const ro_camera *cam, const ro_light *lights, int32_t nlights,
                              const ro_material *mats, int32_t nmats, const ro_sampling *smp, int32_t nthreads,
                              uint8_t *rgb, int32_t *hit_id, float *fimg, int64_t *drawn);

/* Number k that tree node `node` of pixel `pixel` draws (in the
 * reference's order within the node: the lights' rays, then the reflection
 * set, then the refraction set): word k % 4 of Philox4x32-10 with counter
 * (pixel, node low, node high, k / 4) and key (seed low, seed high), as
 * (float)word * 2^-32 -- the reference generator's conversion.  Keyed by
 * node, a subtree's numbers do not depend on how many its elder siblings
 * drew, so subtrees can be traced apart. */
float ro_pixel_stream(uint64_t seed, uint32_t pixel, uint64_t node, uint32_t k);
/* Tree nodes: the camera ray is RO_TREE_ROOT; ray `index` of its
 * reflection (set 0) or refraction (set 1) set is ro_tree_child(node, set,
 * index) = SplitMix64(node + (64 set + index + 1) * 0x9E3779B97F4A7C15). */
#define RO_TREE_ROOT 0x6A09E667F3BCC909ull
uint64_t ro_tree_child(uint64_t parent, int32_t set, int32_t index);

/* n numbers of the reference's random stream (common/common.cc:35-105)
 * from position start of a freshly seeded generator. */
void ro_ref_random(int64_t start, int32_t n, float *out);

/* The reference's cosine table lookups (common/common.h:171-209). */
float ro_lut_cos(float a);
float ro_lut_sin(float a);

/* The AO ray set for one hit (exposed so tests can trace single rays). */
void ro_ao_rays(const float hit_point[3], const float geo_normal[3], uint32_t pixel, int32_t nsamples,
                uint32_t seed, float *ogn, float *dir);

/* Philox4x32-10 (Salmon et al., SC'11) keyed by (key0, key1) on counter ctr. */
void ro_philox4x32(const uint32_t ctr[4], uint32_t key0, uint32_t key1, uint32_t out[4]);

/* Tone-mapping parameters of camera::tone_map (raytracer/camera.h:378):
 * mode is a tone_mapping_mode_t value (camera.h:43-45): 0 none,
 * 1 contrast, 2 local histogram, 3 local histogram with human contrast
 * limits, 4 non-linear, 5 exposure, 6 average luminance, 7 maximum
 * luminance, 9 Ferwerda; key, xw, yw as the reference's arguments;
 * desaturate / stretch its ds / sc flags (glare and temporal adaptation
 * off); gamma > 0 applies camera::gamma_correct(gamma) after.  cam_w,
 * cam_h, cam_t: the camera's half-width, half-height and image-plane
 * distance (the histogram modes resample the frame to one pixel per
 * degree of view). */
typedef struct ro_tone_map {
    int32_t mode;
    float key, xw, yw;
    int32_t desaturate, stretch;
    float gamma;
    float cam_w, cam_h, cam_t;
} ro_tone_map;

/* camera::tone_map (camera.cc:1124-1463) + convert_Yxy_to_rgb
 * (camera.cc:2080-2098) + gamma_correct (camera.cc:1466-1500) in place on a
 * w*h frame of 0..255 colours (3 floats per pixel, index x + y*w).
 * Returns 0, or -1 for an unsupported mode. */
int32_t ro_tone_map_frame(float *img, int32_t w, int32_t h, const ro_tone_map *tm);

#ifdef __cplusplus
}
#endif
#endif
