// raptor_gpu_bvh.h -- drop-in GPU acceleration structure and renderer for
// RAPTor's raytracer, built on the C ABI in include/rtcore.h.
//
// Compiled INSIDE the RAPTor tree: this header includes RAPTor's own
// camera.h, light.h, primitive_store.h, ssd.h and material headers; its one
// source file, raptor_gpu_bvh.cc, joins the raytracer's sources and the
// program links librtcore.so.  Nothing in RAPTor is edited.
//
//   gpu_bvh accel(store)                        <-> bvh accel(store)                 (bvh.h:27-32)
//   accel.find_nearest_object(&ray, &hit)       <-> bvh::find_nearest_object         (bvh.cc:649)
//   accel.found_nearer_object(&ray, t)          <-> bvh::found_nearer_object         (bvh.cc:711)
//   ray_tracer_gpu(&accel, lights, store, cam)  <-> ray_tracer(&accel, lights, store, cam)
//                                                                                  (raytracer.h:105)
//
// ray_tracer_gpu has ray_tracer's signature and effect: every ray of the
// camera's (supersampled) grid is traced and its colour stored with
// camera::set_pixel, so clip_image_to_rgb, tone_map, gamma_correct and the
// image writers then run on the camera unchanged.  It reads the scene from
// the same objects ray_tracer reads: geometry, vertex attributes, vertex
// normals and material pointers of the store's triangles, the lights of the
// light_list and the camera's grid.  Where RAPTor keeps those fields
// private and offers no accessor (light colour and fall-off, material
// coefficients, a triangle's material and vertex data, the camera's grid
// and background), raptor_gpu_bvh.cc reads them through pointers to
// members formed in explicit template instantiations, which C++ exempts
// from access checking ([temp.spec]: "the usual access checking rules do
// not apply to names used to specify explicit instantiations").
//
// Differences a caller sees:
//  - the store is uploaded once, in its current order; ids returned are the
//    store's primitive indices (what primitive_store::indirection returns in
//    the reference), and the store's indirection is left untouched;
//  - single-ray queries each cross the host/device link; batch rays with
//    find_nearest_objects / found_nearer_objects for throughput;
//  - errors throw std::runtime_error carrying rt_last_error_string() (the
//    reference asserts instead);
//  - the GPU path shades coloured_mapper_shader (no texture mappers, or a
//    kd mapper that returns the triangle's per-vertex attribute x 255) and
//    phong_shader without reflection or refraction, up to RT_MAX_MATERIALS
//    distinct materials, point, directional, spot, spherical and
//    triangle-defined lights, a constant background and a pinhole camera;
//    anything else (sky boxes, depth of field, other texture mappers)
//    throws std::invalid_argument naming it;
//  - in a build with SOFT_SHADOW (and DIFFUSE_REFLECTIONS) defined, as the
//    reference's build defines them, frames are rendered as that build
//    renders them (rt_render_distributed): soft shadows draw the
//    reference's random stream from ray_tracer_gpu_stream_position(),
//    which starts at 0 (a fresh program) and moves on by each frame's
//    draws -- a caller that also draws from gen_random_mersenne_twister
//    itself moves it as well; frames with diffuse spreads draw per-pixel
//    streams keyed by ray_tracer_gpu_pixel_seed(), which goes up by one
//    per frame (the reference's single stream cannot be replayed in
//    parallel through diffuse rays).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "camera.h"
#include "light.h"
#include "material.h"
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
rt_context *context(int device = 0);
}  // namespace gpu_detail

class gpu_bvh : public ssd
{
    public :
        // Uploads every triangle of the store (vertices a, b, c; per-vertex
        // attributes and normals where the triangle carries them; light and
        // transparency flags; material index) and builds the GPU hierarchy.
        explicit gpu_bvh(const primitive_store &prims, int device = 0);
        ~gpu_bvh() { rt_scene_destroy(_scene); }
        gpu_bvh(const gpu_bvh &) = delete;
        gpu_bvh &operator=(const gpu_bvh &) = delete;

        // Per-frame update of a simulation loop that keeps the same
        // primitives and moves their vertices (the rebuild at
        // physics_engine/simulation_environment.cc:56-58): refits the
        // existing hierarchy instead of building a new one.
        void refit(const primitive_store &prims);

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

        // The store's distinct materials in order of first use: entry k is
        // material index k of the uploaded triangles.
        const std::vector<const material *> &materials() const { return _materials; }

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
        std::vector<const material *> _materials;
};

// ray_tracer() (raytracer.cc:563-598) on the GPU: same arguments, same
// effect on the camera.  sub_division is used when it is a gpu_bvh built
// from `everything`; any other ssd (a bvh, kd_tree, ...) is replaced by a
// gpu_bvh built from `everything` for this call.
void ray_tracer_gpu(const ssd *const sub_division, const light_list &lights, const primitive_store &everything,
                    camera &c);

// SOFT_SHADOW builds: numbers of the reference's random stream drawn so far
// (the position the next frame's soft shadows start from).
int64_t &ray_tracer_gpu_stream_position();
// DIFFUSE_REFLECTIONS builds: the key of the next frame's per-pixel streams.
uint64_t &ray_tracer_gpu_pixel_seed();
}  // namespace raptor_raytracer
