// raptor_gpu_bvh.h -- drop-in GPU acceleration structure and renderer for
// RAPTor's raytracer, built on the C ABI in include/rtcore.h.
//
// Header-only; compiled INSIDE the RAPTor tree (it includes RAPTor's own
// ssd.h, primitive_store.h, camera.h, light.h and links against
// librtcore.so).  It adds no new interface: a `gpu_bvh` is an `ssd`
// (raytracer/spatial_sub_division/ssd.h:26-44) usable wherever `bvh`, `bih`
// or `kd_tree` is, and `ray_tracer_gpu` takes the arguments of ray_tracer()
// (raytracer/raytracer.h:105).
//
//   gpu_bvh accel(primitive_store&)             <-> bvh accel(primitive_store&)
//   accel.find_nearest_object(&ray, &hit)       <-> bvh::find_nearest_object (bvh.cc:649)
//   accel.found_nearer_object(&ray, t)          <-> bvh::found_nearer_object (bvh.cc:711)
//   ray_tracer_gpu(&accel, lights, cam_args,   <-> ray_tracer(&accel, lights, store, cam)
//                  cam, ka, kd, ks, ns, colours)   (raytracer.cc:563)
//
// Differences a caller sees:
//  - the store is uploaded once, in its current order; ids returned are the
//    store's primitive indices (what primitive_store::indirection returns in
//    the reference), and the store's indirection is left untouched;
//  - single-ray queries each cross the PCIe/C2C link; batch rays with
//    find_nearest_objects / found_nearer_objects for throughput;
//  - errors throw std::runtime_error carrying rt_last_error_string() (the
//    reference asserts instead);
//  - ray_tracer_gpu shades with the coloured Phong model of
//    coloured_mapper_shader (ka, kd, ks, ns; kd modulated by a per-vertex
//    colour), the only material on the GPU path.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "camera.h"
#include "light.h"
#include "primitive_store.h"
#include "ssd.h"

#include "rtcore.h"

namespace raptor_raytracer
{
namespace gpu_detail
{
inline void check(rt_status s)
{
    if (s != RT_OK) throw std::runtime_error(std::string("rtcore: ") + rt_last_error_string());
}

// One process-wide context per device (created on first use).
inline rt_context *context(int device = 0)
{
    static rt_context *ctx = nullptr;
    if (!ctx) check(rt_ctx_create(device, &ctx));
    return ctx;
}
}  // namespace gpu_detail

class gpu_bvh : public ssd
{
    public :
        // Uploads every triangle of the store (vertices a, b, c; light flag;
        // transparency) and builds the GPU hierarchy.
        explicit gpu_bvh(const primitive_store &prims, int device = 0) : _scene(nullptr)
        {
            gpu_detail::check(rt_scene_create(gpu_detail::context(device), &_scene));
            const int n = prims.size();
            std::vector<float> verts(9 * (size_t)n);
            std::vector<int32_t> idx(3 * (size_t)n);
            std::vector<uint32_t> flags((size_t)n);
            for (int i = 0; i < n; ++i)
            {
                const triangle *t = prims.primitive(i);
                const point_t<> v[3] = { t->get_vertex_a(), t->get_vertex_b(), t->get_vertex_c() };
                for (int k = 0; k < 3; ++k)
                {
                    verts[9 * i + 3 * k + 0] = v[k].x;
                    verts[9 * i + 3 * k + 1] = v[k].y;
                    verts[9 * i + 3 * k + 2] = v[k].z;
                    idx[3 * i + k] = 3 * i + k;
                }
                flags[i] = (t->get_light() ? RT_TRI_LIGHT : 0u) | (t->is_transparent() ? RT_TRI_TRANSPARENT : 0u);
            }
            gpu_detail::check(rt_scene_upload(_scene, verts.data(), 3 * n, idx.data(), n, nullptr, flags.data()));
            gpu_detail::check(rt_bvh_build(_scene, nullptr));
        }

        // Per-frame update of a simulation loop that keeps the same
        // primitives and moves their vertices (the rebuild at
        // physics_engine/simulation_environment.cc:56-58): refits the
        // existing hierarchy instead of building a new one.
        void refit(const primitive_store &prims)
        {
            const int n = prims.size();
            std::vector<float> verts(9 * (size_t)n);
            for (int i = 0; i < n; ++i)
            {
                const triangle *t = prims.primitive(i);
                const point_t<> v[3] = { t->get_vertex_a(), t->get_vertex_b(), t->get_vertex_c() };
                for (int k = 0; k < 3; ++k)
                {
                    verts[9 * i + 3 * k + 0] = v[k].x;
                    verts[9 * i + 3 * k + 1] = v[k].y;
                    verts[9 * i + 3 * k + 2] = v[k].z;
                }
            }
            gpu_detail::check(rt_scene_refit_vertices(_scene, verts.data(), 3 * n, nullptr));
        }

        ~gpu_bvh() { rt_scene_destroy(_scene); }
        gpu_bvh(const gpu_bvh &) = delete;
        gpu_bvh &operator=(const gpu_bvh &) = delete;

        // ssd interface: one ray per call.
        int find_nearest_object(const ray *const r, hit_description *const h) const override
        {
            rt_hit out;
            const rt_ray q = to_rt(*r, 0.0f);
            gpu_detail::check(rt_trace_closest(_scene, &q, 1, &out));
            *h = hit_description(out.t, hit_t::miss, out.u, out.v);
            return out.tri;
        }

        bool found_nearer_object(const ray *const r, const float t) const override
        {
            uint8_t occ = 0;
            const rt_ray q = to_rt(*r, t);
            gpu_detail::check(rt_trace_any(_scene, &q, 1, &occ));
            return occ != 0;
        }

        // Batched forms of the two queries (same semantics, n rays per call).
        void find_nearest_objects(const ray *const r, const int n, int *const ids, hit_description *const h) const
        {
            std::vector<rt_ray> q((size_t)n);
            std::vector<rt_hit> out((size_t)n);
            for (int i = 0; i < n; ++i) q[i] = to_rt(r[i], 0.0f);
            gpu_detail::check(rt_trace_closest(_scene, q.data(), n, out.data()));
            for (int i = 0; i < n; ++i)
            {
                ids[i] = out[i].tri;
                h[i] = hit_description(out[i].t, hit_t::miss, out[i].u, out[i].v);
            }
        }

        void found_nearer_objects(const ray *const r, const float *const t, const int n, bool *const occluded) const
        {
            std::vector<rt_ray> q((size_t)n);
            std::vector<uint8_t> out((size_t)n);
            for (int i = 0; i < n; ++i) q[i] = to_rt(r[i], t[i]);
            gpu_detail::check(rt_trace_any(_scene, q.data(), n, out.data()));
            for (int i = 0; i < n; ++i) occluded[i] = out[i] != 0;
        }

        rt_scene *scene() const { return _scene; }

    private :
        static rt_ray to_rt(const ray &r, const float tmax)
        {
            const point_t<> o = r.get_ogn(), d = r.get_dir();
            rt_ray q;
            q.ox = o.x; q.oy = o.y; q.oz = o.z; q.tmax = tmax;
            q.dx = d.x; q.dy = d.y; q.dz = d.z; q.pad = 0.0f;
            return q;
        }

        rt_scene *_scene;
};

// Camera arguments of the reference camera constructor (camera.h:55-62):
// the renderer needs them explicitly because camera keeps them private.
struct gpu_camera_args
{
    point_t<> position, x_axis, y_axis, z_axis;
    ext_colour_t background;
    float w, h, t;
    unsigned x_res, y_res;
};

struct gpu_light_args
{
    bool directional;
    ext_colour_t rgb;      /* 0..255 */
    point_t<> centre;      /* point and spot light */
    point_t<> direction;   /* directional light; a spot light's n */
    float d;
    float s_a = 0.0f, s_b = 0.0f;   /* spot light cone (light.h:24-25); s_b = 0: not a spot light */
};

// ray_tracer() replacement: renders the frame on the GPU and writes every
// pixel through camera::set_pixel (camera.h:281), so clip_image_to_rgb and
// the image writers work unchanged.  vertex_colours: 3 floats per vertex of
// the store in triangle order (a, b, c of triangle 0, then triangle 1, ...),
// nullable.  rf, tran, ri: the material's reflectivity, transparency and
// refractive index (coloured_mapper_shader's rf, tran, ri).
inline void ray_tracer_gpu(const gpu_bvh *const accel, const std::vector<gpu_light_args> &lights,
                           const gpu_camera_args &cam_args, camera &c, const ext_colour_t &ka, const ext_colour_t &kd,
                           const ext_colour_t &ks, const float ns, const float *vertex_colours = nullptr,
                           const float rf = 0.0f, const float tran = 0.0f, const float ri = 1.0f)
{
    rt_camera cam;
    const point_t<> *ax[4] = { &cam_args.position, &cam_args.x_axis, &cam_args.y_axis, &cam_args.z_axis };
    float *dst[4] = { cam.pos, cam.x_axis, cam.y_axis, cam.z_axis };
    for (int i = 0; i < 4; ++i) { dst[i][0] = ax[i]->x; dst[i][1] = ax[i]->y; dst[i][2] = ax[i]->z; }
    cam.background[0] = cam_args.background.r; cam.background[1] = cam_args.background.g; cam.background[2] = cam_args.background.b;
    cam.w = cam_args.w; cam.h = cam_args.h; cam.t = cam_args.t;
    cam.xres = (int32_t)cam_args.x_res; cam.yres = (int32_t)cam_args.y_res;
    std::vector<rt_light> ls(lights.size());
    for (size_t i = 0; i < lights.size(); ++i)
    {
        const gpu_light_args &l = lights[i];
        ls[i].kind = l.directional ? RT_LIGHT_DIRECTIONAL : RT_LIGHT_POINT;
        ls[i].rgb[0] = l.rgb.r; ls[i].rgb[1] = l.rgb.g; ls[i].rgb[2] = l.rgb.b;
        ls[i].pos[0] = l.centre.x; ls[i].pos[1] = l.centre.y; ls[i].pos[2] = l.centre.z;
        ls[i].dir[0] = l.direction.x; ls[i].dir[1] = l.direction.y; ls[i].dir[2] = l.direction.z;
        ls[i].d = l.d;
        if (!l.directional && l.s_b != 0.0f) ls[i].kind = RT_LIGHT_SPOT;
        ls[i].s_a = l.s_a;
        ls[i].s_b = l.s_b;
    }
    rt_material m;
    m.ka[0] = ka.r; m.ka[1] = ka.g; m.ka[2] = ka.b;
    m.kd[0] = kd.r; m.kd[1] = kd.g; m.kd[2] = kd.b;
    m.ks[0] = ks.r; m.ks[1] = ks.g; m.ks[2] = ks.b;
    m.ns = ns;
    m.rf = rf;
    m.tran = tran;
    m.ri = ri;
    m.flags = 0u;
    rt_scene *s = accel->scene();
    if (vertex_colours)
    {
        int32_t nodes, tris, depth;
        gpu_detail::check(rt_bvh_info(s, &nodes, &tris, &depth));
        gpu_detail::check(rt_scene_update_attributes(s, vertex_colours, 3 * tris));
    }
    const size_t npix = (size_t)cam.xres * (size_t)cam.yres;
    std::vector<uint8_t> rgb(3 * npix);
    gpu_detail::check(rt_render(s, &cam, ls.data(), (int32_t)ls.size(), &m, rgb.data(), nullptr, nullptr));
    for (unsigned y = 0; y < cam_args.y_res; ++y)
        for (unsigned x = 0; x < cam_args.x_res; ++x)
        {
            const size_t p = 3 * ((size_t)x + (size_t)y * cam_args.x_res);
            c.set_pixel(ext_colour_t(rgb[p], rgb[p + 1], rgb[p + 2]), x, y);
        }
}
}  // namespace raptor_raytracer
