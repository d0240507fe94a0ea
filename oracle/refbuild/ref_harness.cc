// ref_harness.cc -- drives the UNMODIFIED RAPTor sources (compiled from the
// reference tree by oracle/refbuild/Makefile) through their own public API,
// so tests can pin the C restatement in oracle/rtoracle.c against the
// reference itself and generate golden fixtures.
//
// TEST INFRASTRUCTURE ONLY.  Builds only on x86-64 hosts: the reference's
// common/simd.h includes <immintrin.h> unconditionally.
//
// Entry points mirror oracle/rtoracle.h one for one (prefix rref_).
#include <cstdint>
#include <cstring>
#include <chrono>
#include <iostream>
#include <memory>
#include <streambuf>
#include <vector>

#include <fstream>
#include <list>

#include "bvh.h"
#include "camera.h"
#include "coloured_mapper_shader.h"
#include "light.h"
#include "primitive_store.h"
#include "raytracer.h"
#include "texture_mapper.h"
#include "obj_parser.h"
#include "off_parser.h"
#include "ply_parser.h"

#include "../rtoracle.h"

using namespace raptor_raytracer;

namespace {

// Texture mapper that returns the interpolated per-vertex attribute scaled
// to 0..255, which is how a per-vertex colour reaches
// coloured_mapper_shader::shade (coloured_mapper_shader.cc:61-66).
class vertex_colour_mapper : public texture_mapper {
  protected:
    float sample_texture(const ray &, ext_colour_t *const c, const point_t<> &, const point_t<> &vt) const override
    {
        *c = ext_colour_t(vt.x * 255.0f, vt.y * 255.0f, vt.z * 255.0f);
        return 1.0f;
    }
    float sample_texture_monochrome(const ray &, point_t<> *const p, const point_t<> &, const point_t<> &vt,
                                    const int, const int) const override
    {
        p->z = vt.x * 255.0f;
        return 1.0f;
    }
};

struct null_buf : std::streambuf {
    int overflow(int c) override { return c; }
    std::streamsize xsputn(const char *, std::streamsize n) override { return n; }
};

struct ref_scene {
    std::unique_ptr<material> opaque;
    std::unique_ptr<material> transparent;
    std::vector<std::unique_ptr<material>> table;
    primitive_store store;
    std::unique_ptr<bvh> accel;
};

point_t<> p3(const float *p) { return point_t<>(p[0], p[1], p[2]); }

}  // namespace

extern "C" {

void *rref_scene_create(const float *verts, int32_t nverts, const int32_t *tris, int32_t ntris, const float *vattr,
                        const uint32_t *flags, const ro_material *m)
{
    (void)nverts;
    auto *s = new ref_scene();
    const texture_mapper *kd_map = vattr ? new vertex_colour_mapper() : nullptr;
    s->opaque.reset(new coloured_mapper_shader(ext_colour_t(m->ka[0], m->ka[1], m->ka[2]),
                                               ext_colour_t(m->kd[0], m->kd[1], m->kd[2]),
                                               ext_colour_t(m->ks[0], m->ks[1], m->ks[2]), m->ns, 0.0f, 1.0f, m->rf,
                                               0.0f, m->rfd, nullptr, kd_map));
    s->transparent.reset(new coloured_mapper_shader(ext_colour_t(m->ka[0], m->ka[1], m->ka[2]),
                                                    ext_colour_t(m->kd[0], m->kd[1], m->kd[2]),
                                                    ext_colour_t(m->ks[0], m->ks[1], m->ks[2]), m->ns, 0.5f, 1.0f));
    s->store.reserve(ntris);
    for (int32_t i = 0; i < ntris; ++i) {
        const int32_t ia = tris[3 * i], ib = tris[3 * i + 1], ic = tris[3 * i + 2];
        const uint32_t f = flags ? flags[i] : 0u;
        material *mat = (f & RO_TRI_TRANSPARENT) ? s->transparent.get() : s->opaque.get();
        if (vattr) {
            point_t<> vt[3] = {p3(vattr + 3 * ia), p3(vattr + 3 * ib), p3(vattr + 3 * ic)};
            s->store.emplace_back(mat, p3(verts + 3 * ia), p3(verts + 3 * ib), p3(verts + 3 * ic),
                                  (f & RO_TRI_LIGHT) != 0, static_cast<const point_t<> *>(nullptr),
                                  static_cast<const point_t<> *>(vt));
        } else {
            s->store.emplace_back(mat, p3(verts + 3 * ia), p3(verts + 3 * ib), p3(verts + 3 * ic),
                                  (f & RO_TRI_LIGHT) != 0);
        }
    }
    return s;
}

// A scene whose triangles carry per-triangle materials from a table (the
// reference's material pointer per triangle, triangle.h:99-106): one
// coloured_mapper_shader per entry with its tran, ri, rf, td and rfd; kd
// follows the vertex colour unless the entry says otherwise.
void *rref_scene_create_mt(const float *verts, int32_t nverts, const int32_t *tris, int32_t ntris, const float *vattr,
                           const uint32_t *flags, const ro_material *mats, int32_t nmats, const int32_t *mat_of_tri)
{
    (void)nverts;
    auto *s = new ref_scene();
    for (int32_t k = 0; k < nmats; ++k) {
        const ro_material *m = &mats[k];
        // each shader owns (and deletes) its texture mappers: one per entry
        const texture_mapper *map =
            (vattr && !(m->flags & RO_MAT_NO_VERTEX_COLOUR)) ? new vertex_colour_mapper() : nullptr;
        s->table.emplace_back(new coloured_mapper_shader(ext_colour_t(m->ka[0], m->ka[1], m->ka[2]),
                                                         ext_colour_t(m->kd[0], m->kd[1], m->kd[2]),
                                                         ext_colour_t(m->ks[0], m->ks[1], m->ks[2]), m->ns, m->tran,
                                                         m->ri, m->rf, m->td, m->rfd, nullptr, map));
    }
    s->store.reserve(ntris);
    for (int32_t i = 0; i < ntris; ++i) {
        const int32_t ia = tris[3 * i], ib = tris[3 * i + 1], ic = tris[3 * i + 2];
        const uint32_t f = flags ? flags[i] : 0u;
        material *mat = s->table[mat_of_tri ? mat_of_tri[i] : 0].get();
        if (vattr) {
            point_t<> vt[3] = {p3(vattr + 3 * ia), p3(vattr + 3 * ib), p3(vattr + 3 * ic)};
            s->store.emplace_back(mat, p3(verts + 3 * ia), p3(verts + 3 * ib), p3(verts + 3 * ic),
                                  (f & RO_TRI_LIGHT) != 0, static_cast<const point_t<> *>(nullptr),
                                  static_cast<const point_t<> *>(vt));
        } else {
            s->store.emplace_back(mat, p3(verts + 3 * ia), p3(verts + 3 * ib), p3(verts + 3 * ic),
                                  (f & RO_TRI_LIGHT) != 0);
        }
    }
    return s;
}

double rref_scene_build(void *h)
{
    auto *s = static_cast<ref_scene *>(h);
    const auto t0 = std::chrono::steady_clock::now();
    s->accel.reset(new bvh(s->store));
    const auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

void rref_scene_destroy(void *h) { delete static_cast<ref_scene *>(h); }

int32_t rref_trace_closest(void *h, const float *ogn, const float *dir, int32_t n, int32_t *id, float *t, float *u,
                           float *v)
{
    auto *s = static_cast<ref_scene *>(h);
    for (int32_t i = 0; i < n; ++i) {
        const ray r(p3(ogn + 3 * i), dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
        hit_description hd;
        id[i] = s->accel->find_nearest_object(&r, &hd);
        t[i] = hd.d;
        if (u) u[i] = hd.u;
        if (v) v[i] = hd.v;
    }
    return 0;
}

int32_t rref_trace_any(void *h, const float *ogn, const float *dir, const float *tmax, int32_t n, uint8_t *occ)
{
    auto *s = static_cast<ref_scene *>(h);
    for (int32_t i = 0; i < n; ++i) {
        const ray r(p3(ogn + 3 * i), dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
        occ[i] = s->accel->found_nearer_object(&r, tmax[i]) ? 1 : 0;
    }
    return 0;
}

static camera *make_camera(const ro_camera *c, unsigned aa_x = 1u, unsigned aa_y = 1u)
{
    return new camera(p3(c->pos), p3(c->x_axis), p3(c->y_axis), p3(c->z_axis),
                      ext_colour_t(c->background[0], c->background[1], c->background[2]), c->w, c->h, c->t,
                      (unsigned)c->xres, (unsigned)c->yres, aa_x, aa_y, 0.0f, 0.0f);
}

void rref_camera_rays(const ro_camera *c, int32_t x0, int32_t y0, int32_t w, int32_t hgt, float *ogn, float *dir)
{
    std::unique_ptr<camera> cam(make_camera(c));
    std::vector<ray> rays;
    size_t k = 0;
    for (int32_t y = y0; y < y0 + hgt; ++y)
        for (int32_t x = x0; x < x0 + w; ++x, ++k) {
            cam->pixel_to_co_ordinate(&rays, x, y, 1, 1, 16);
            const point_t<> o = rays[0].get_ogn(), d = rays[0].get_dir();
            ogn[3 * k] = o.x; ogn[3 * k + 1] = o.y; ogn[3 * k + 2] = o.z;
            dir[3 * k] = d.x; dir[3 * k + 1] = d.y; dir[3 * k + 2] = d.z;
        }
}

// Full-frame render through ray_tracer() (raytracer.cc:563) and
// clip_image_to_rgb (camera.h:289).  The per-pixel progress line the
// reference prints (raytracer.cc:529) goes to a null stream.  Returns the
// render wall time in seconds.
// The same with anti-aliasing: the camera traces aa_x * aa_y rays per output
// pixel (camera.h:55-62, x_a_res / y_a_res) and clip_image_to_rgb averages
// them (camera.h:289-319).  rgb holds xres * yres output pixels.
double rref_render_aa(void *h, const ro_camera *c, int32_t aa_x, int32_t aa_y, const ro_light *ls, int32_t nl,
                      uint8_t *rgb);

// The caller's lights as the reference's light objects: directional
// (light.h:33-34), spot (light.h:24-25), spherical (light.h:17-18), or
// defined by triangles of the store (light.h:20-21, spot form :27-29).
// tri_lists keeps the lists those lights point to alive.
static void make_lights(const ro_light *ls, int32_t nl, const primitive_store *store, light_list &lights,
                        std::vector<std::vector<int>> &tri_lists)
{
    tri_lists.reserve((size_t)(nl > 0 ? nl : 0));
    for (int32_t i = 0; i < nl; ++i) {
        const ext_colour_t rgbc(ls[i].rgb[0], ls[i].rgb[1], ls[i].rgb[2]);
        if (ls[i].kind == 1) {
            lights.emplace_back(rgbc, p3(ls[i].dir), ls[i].d);
        } else if (ls[i].ntris > 0 && ls[i].tris) {
            tri_lists.emplace_back(ls[i].tris, ls[i].tris + ls[i].ntris);
            const std::vector<int> *t = &tri_lists.back();
            if (ls[i].kind == 2)
                lights.emplace_back(store, rgbc, p3(ls[i].pos), p3(ls[i].dir), ls[i].d, ls[i].s_a, ls[i].s_b, t);
            else
                lights.emplace_back(store, rgbc, p3(ls[i].pos), ls[i].d, t);
        } else if (ls[i].kind == 2) {
            lights.emplace_back(rgbc, p3(ls[i].pos), p3(ls[i].dir), ls[i].d, ls[i].s_a, ls[i].s_b, ls[i].r);
        } else {
            lights.emplace_back(rgbc, p3(ls[i].pos), ls[i].d, ls[i].r);
        }
    }
}

double rref_render(void *h, const ro_camera *c, const ro_light *ls, int32_t nl, uint8_t *rgb)
{
    return rref_render_aa(h, c, 1, 1, ls, nl, rgb);
}

// The frame of rref_render_aa, tone mapped by the reference's
// camera::tone_map (camera.cc:1124) with glare and temporal adaptation off,
// then camera::gamma_correct (camera.cc:1466) when tm->gamma > 0, before
// clip_image_to_rgb.  tm NULL: neither.
double rref_render_tone_mapped(void *h, const ro_camera *c, int32_t aa_x, int32_t aa_y, const ro_light *ls,
                               int32_t nl, const ro_tone_map *tm, uint8_t *rgb)
{
    auto *s = static_cast<ref_scene *>(h);
    std::unique_ptr<camera> cam(make_camera(c, (unsigned)aa_x, (unsigned)aa_y));
    light_list lights;
    std::vector<std::vector<int>> tri_lists;
    make_lights(ls, nl, &s->store, lights, tri_lists);
    null_buf nb;
    std::streambuf *old = std::cout.rdbuf(&nb);
    const auto t0 = std::chrono::steady_clock::now();
    ray_tracer(s->accel.get(), lights, s->store, *cam);
    if (tm) {
        cam->tone_map(static_cast<tone_mapping_mode_t>(tm->mode), tm->key, tm->xw, tm->yw, false, false,
                      tm->desaturate != 0, tm->stretch != 0);
        if (tm->gamma > 0.0f) cam->gamma_correct(tm->gamma);
    }
    const auto t1 = std::chrono::steady_clock::now();
    std::cout.rdbuf(old);
    cam->clip_image_to_rgb(rgb);
    return std::chrono::duration<double>(t1 - t0).count();
}

// The reference's tone mapping alone: a camera of c's geometry (aa_x * aa_y
// samples per output pixel) whose image is set to fimg (3 floats per
// sample of the supersampled grid, row y = 0 first) through
// camera::set_pixel, then tone_map + gamma_correct as above and
// clip_image_to_rgb.
void rref_tone_map_image(const ro_camera *c, int32_t aa_x, int32_t aa_y, const float *fimg, const ro_tone_map *tm,
                         uint8_t *rgb)
{
    std::unique_ptr<camera> cam(make_camera(c, (unsigned)aa_x, (unsigned)aa_y));
    const int32_t fw = c->xres * aa_x, fh = c->yres * aa_y;
    for (int32_t y = 0; y < fh; ++y)
        for (int32_t x = 0; x < fw; ++x) {
            const float *p = fimg + 3 * ((size_t)y * fw + x);
            cam->set_pixel(ext_colour_t(p[0], p[1], p[2]), x, y);
        }
    cam->tone_map(static_cast<tone_mapping_mode_t>(tm->mode), tm->key, tm->xw, tm->yw, false, false,
                  tm->desaturate != 0, tm->stretch != 0);
    if (tm->gamma > 0.0f) cam->gamma_correct(tm->gamma);
    cam->clip_image_to_rgb(rgb);
}

double rref_render_aa(void *h, const ro_camera *c, int32_t aa_x, int32_t aa_y, const ro_light *ls, int32_t nl,
                      uint8_t *rgb)
{
    return rref_render_tone_mapped(h, c, aa_x, aa_y, ls, nl, nullptr, rgb);
}

int32_t rref_morton_code(float x, float y, float z, float xm, float ym, float zm)
{
    return morton_code(x, y, z, xm, ym, zm);
}

// A mesh file through the reference's own parser (off_parser.cc /
// ply_parser.cc / obj_parser.cc; kind 1 OFF, 2 PLY, 3 OBJ): the vertices of each primitive in
// primitive_store order (9 floats per triangle, at most max_tris written)
// and the number of materials the parser made (*nmat).  Returns the
// triangle count, or -1 if the file cannot be opened.
int64_t rref_parse_mesh(const char *path, int32_t kind, float *tri_out, int64_t max_tris, int32_t *nmat)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return -1;
    light_list lights;
    primitive_store store;
    std::list<material *> mats;
    if (kind == 1) {
        off_parser(f, lights, store, mats, nullptr);
    } else if (kind == 3) {
        camera *cam = nullptr;
        obj_parser(f, std::string(""), lights, store, mats, &cam);
    } else {
        camera *cam = nullptr;
        ply_parser(f, lights, store, mats, &cam);
    }
    const int64_t n = (int64_t)store.size();
    for (int64_t i = 0; i < n && i < max_tris; ++i) {
        const triangle *t = store.primitive((int)i);
        const point_t<> v[3] = {t->get_vertex_a(), t->get_vertex_b(), t->get_vertex_c()};
        for (int k = 0; k < 3; ++k) {
            tri_out[9 * i + 3 * k] = v[k].x;
            tri_out[9 * i + 3 * k + 1] = v[k].y;
            tri_out[9 * i + 3 * k + 2] = v[k].z;
        }
    }
    *nmat = (int32_t)mats.size();
    for (material *m : mats) delete m;
    return n;
}

// A mesh file parsed by the reference's own parser (kind 1 OFF, 2 PLY,
// 3 OBJ) with the materials it creates (phong_shader), then rendered by
// ray_tracer and clip_image_to_rgb.  Returns the triangle count, or -1.
int64_t rref_parse_and_render(const char *path, int32_t kind, const ro_camera *c, const ro_light *ls, int32_t nl,
                              uint8_t *rgb)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return -1;
    light_list parsed_lights;
    primitive_store store;
    std::list<material *> mats;
    camera *cam_unused = nullptr;
    if (kind == 1) off_parser(f, parsed_lights, store, mats, nullptr);
    else if (kind == 3) obj_parser(f, std::string(""), parsed_lights, store, mats, &cam_unused);
    else ply_parser(f, parsed_lights, store, mats, &cam_unused);
    const int64_t n = (int64_t)store.size();
    {
        std::unique_ptr<bvh> accel(new bvh(store));
        std::unique_ptr<camera> cam(make_camera(c));
        light_list lights;
        std::vector<std::vector<int>> tri_lists;
        make_lights(ls, nl, &store, lights, tri_lists);
        null_buf nb;
        std::streambuf *old = std::cout.rdbuf(&nb);
        ray_tracer(accel.get(), lights, store, *cam);
        std::cout.rdbuf(old);
        cam->clip_image_to_rgb(rgb);
    }
    for (material *m : mats) delete m;
    return n;
}

// The reference's own random stream (common/common.cc:35-105): the next n
// numbers of the process-wide generator, which soft shadows draw from.
void rref_random(int32_t n, float *out)
{
    for (int32_t i = 0; i < n; ++i) out[i] = gen_random_mersenne_twister();
}

// The reference's cosine table (common.h:171-209) as light::find_rays reads it.
float rref_lut_cos(float a) { return cos_lut.get_cos(a); }
float rref_lut_sin(float a) { return cos_lut.get_sin(a); }

// Shadow rays per light of a primary hit in this build (SOFT_SHADOW, or 1).
int32_t rref_soft_shadow_samples(void) { return SHADOW_ARRAY_SIZE; }

// Rays of a diffuse reflection of a primary hit in this build
// (DIFFUSE_REFLECTIONS, or 0 when it is off).
int32_t rref_diffuse_samples(void)
{
#ifdef DIFFUSE_REFLECTIONS
    return MAX_SECONDARY_RAYS;
#else
    return 0;
#endif
}

}  // extern "C"
