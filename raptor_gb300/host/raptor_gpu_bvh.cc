// raptor_gpu_bvh.cc -- the scene hand-over of raptor_gpu_bvh.h: RAPTor's
// triangles, lights, materials and camera turned into the C ABI's arrays and
// structs, and ray_tracer_gpu.  Compiled once, inside the RAPTor tree.
#include "raptor_gpu_bvh.h"

#include <cfloat>
#include <cmath>
#include <map>
#include <memory>

#include "coloured_mapper_shader.h"
#include "phong_shader.h"

namespace raptor_raytracer
{
namespace gpu_detail
{
rt_context *context(int device)
{
    static std::map<int, rt_context *> ctx;
    rt_context *&c = ctx[device];
    if (!c) check(rt_ctx_create(device, &c));
    return c;
}

// ---------------------------------------------------------------------
// Read access to data members RAPTor keeps private.  An explicit
// instantiation may name a private member (access checking does not apply
// to the names in an explicit instantiation); the pointer to member it is
// given is returned by a friend function, found by argument-dependent
// lookup on the tag type.  Reads only; the objects are never modified.
template <typename Tag, typename Tag::type Member>
struct member_of
{
    friend typename Tag::type member(Tag) { return Member; }
};

#define RAPTOR_GPU_MEMBER(TAG, CLASS, TYPE, NAME)   \
    struct TAG                                       \
    {                                                \
        typedef TYPE CLASS::*type;                   \
        friend type member(TAG);                     \
    };                                               \
    template struct member_of<TAG, &CLASS::NAME>;

// camera (camera.h:520-555) and base_camera (sdl_wrappers/base_camera.h:111-116)
RAPTOR_GPU_MEMBER(cam_tm, camera, const std::vector<texture_mapper *> *const, tm)
RAPTOR_GPU_MEMBER(cam_b, camera, const ext_colour_t, b)
RAPTOR_GPU_MEMBER(cam_x_m, camera, const float, x_m)
RAPTOR_GPU_MEMBER(cam_y_m, camera, const float, y_m)
RAPTOR_GPU_MEMBER(cam_t, camera, const float, t)
RAPTOR_GPU_MEMBER(cam_x_res, camera, const unsigned, x_res)
RAPTOR_GPU_MEMBER(cam_y_res, camera, const unsigned, y_res)
RAPTOR_GPU_MEMBER(cam_aperture, camera, float, aperture)
RAPTOR_GPU_MEMBER(cam_focal_length, camera, float, focal_length)
RAPTOR_GPU_MEMBER(bcam_x, base_camera, point_t<>, _x)
RAPTOR_GPU_MEMBER(bcam_y, base_camera, point_t<>, _y)
RAPTOR_GPU_MEMBER(bcam_z, base_camera, point_t<>, _z)
// light (light.h:203-213)
RAPTOR_GPU_MEMBER(light_rgb, light, const ext_colour_t, rgb)
RAPTOR_GPU_MEMBER(light_n, light, const point_t<>, n)
RAPTOR_GPU_MEMBER(light_d, light, const float, d)
RAPTOR_GPU_MEMBER(light_s_a, light, const float, s_a)
RAPTOR_GPU_MEMBER(light_s_b, light, const float, s_b)
RAPTOR_GPU_MEMBER(light_r, light, const float, r)
RAPTOR_GPU_MEMBER(light_t, light, const std::vector<int> *const, t)
// triangle (triangle.h:100-112)
RAPTOR_GPU_MEMBER(tri_m, triangle, std::int64_t, m)
RAPTOR_GPU_MEMBER(tri_vnt, triangle, point_t<> *, vnt)
// coloured_mapper_shader (coloured_mapper_shader.h:91-107)
RAPTOR_GPU_MEMBER(cms_t_ka, coloured_mapper_shader, const texture_mapper *, t_ka)
RAPTOR_GPU_MEMBER(cms_t_kd, coloured_mapper_shader, const texture_mapper *, t_kd)
RAPTOR_GPU_MEMBER(cms_t_ks, coloured_mapper_shader, const texture_mapper *, t_ks)
RAPTOR_GPU_MEMBER(cms_t_ns, coloured_mapper_shader, const texture_mapper *, t_ns)
RAPTOR_GPU_MEMBER(cms_t_refl, coloured_mapper_shader, const texture_mapper *, t_refl)
RAPTOR_GPU_MEMBER(cms_t_d, coloured_mapper_shader, const texture_mapper *, t_d)
RAPTOR_GPU_MEMBER(cms_ka, coloured_mapper_shader, const ext_colour_t, ka)
RAPTOR_GPU_MEMBER(cms_kd, coloured_mapper_shader, const ext_colour_t, kd)
RAPTOR_GPU_MEMBER(cms_ks, coloured_mapper_shader, const ext_colour_t, ks)
RAPTOR_GPU_MEMBER(cms_ns, coloured_mapper_shader, const float, ns)
RAPTOR_GPU_MEMBER(cms_tran, coloured_mapper_shader, const float, tran)
RAPTOR_GPU_MEMBER(cms_ri, coloured_mapper_shader, const float, ri)
RAPTOR_GPU_MEMBER(cms_rf, coloured_mapper_shader, const float, rf)
RAPTOR_GPU_MEMBER(cms_td, coloured_mapper_shader, const float, td)
RAPTOR_GPU_MEMBER(cms_rfd, coloured_mapper_shader, const float, rfd)
// phong_shader (phong_shader.h:66-75)
RAPTOR_GPU_MEMBER(ps_ka, phong_shader, const ext_colour_t, ka)
RAPTOR_GPU_MEMBER(ps_kd, phong_shader, const ext_colour_t, kd)
RAPTOR_GPU_MEMBER(ps_ks, phong_shader, const ext_colour_t, ks)
RAPTOR_GPU_MEMBER(ps_s, phong_shader, const float, s)
RAPTOR_GPU_MEMBER(ps_tran, phong_shader, const float, tran)
RAPTOR_GPU_MEMBER(ps_rf, phong_shader, const float, rf)
RAPTOR_GPU_MEMBER(ps_td, phong_shader, const float, td)
RAPTOR_GPU_MEMBER(ps_rfd, phong_shader, const float, rfd)

#undef RAPTOR_GPU_MEMBER

template <typename Tag, typename Obj>
auto field(const Obj &o, Tag tag) -> decltype(o.*member(tag))
{
    return o.*member(tag);
}

void unsupported(const std::string &what)
{
    throw std::invalid_argument("ray_tracer_gpu: " + what + " is not supported on the GPU path");
}

// The material pointer of a triangle (its light flag in bit 0 removed,
// triangle.h:99-103).
const material *material_of(const triangle &t)
{
    return reinterpret_cast<const material *>(field(t, tri_m{}) & ~std::int64_t(1));
}

void put3(float *dst, const point_t<> &p)
{
    dst[0] = p.x;
    dst[1] = p.y;
    dst[2] = p.z;
}

void put3(float *dst, const ext_colour_t &c)
{
    dst[0] = c.r;
    dst[1] = c.g;
    dst[2] = c.b;
}

// rt_material of a RAPTor material (coloured_mapper_shader::shade,
// coloured_mapper_shader.cc:41-115; phong_shader::shade, phong_shader.cc:21-64).
rt_material describe(const material *m)
{
    rt_material out;
    if (const coloured_mapper_shader *c = dynamic_cast<const coloured_mapper_shader *>(m))
    {
        if (field(*c, cms_t_ka{}) || field(*c, cms_t_ks{}) || field(*c, cms_t_ns{}) || field(*c, cms_t_refl{}) ||
            field(*c, cms_t_d{}))
            unsupported("a coloured_mapper_shader texture mapper other than kd's");
        put3(out.ka, field(*c, cms_ka{}));
        put3(out.kd, field(*c, cms_kd{}));
        put3(out.ks, field(*c, cms_ks{}));
        out.ns = field(*c, cms_ns{});
        out.rf = field(*c, cms_rf{});
        out.tran = field(*c, cms_tran{});
        out.ri = field(*c, cms_ri{});
        // spreads of diffuse reflection and refraction: a build without
        // DIFFUSE_REFLECTIONS ignores them (ray.cc:118-135, 198-235), as the
        // renders ray_tracer_gpu uses do
        out.rfd = field(*c, cms_rfd{});
        out.td = field(*c, cms_td{});
        // a kd texture mapper samples the triangle's per-vertex attribute
        out.flags = field(*c, cms_t_kd{}) ? 0u : RT_MAT_NO_VERTEX_COLOUR;
        return out;
    }
    if (const phong_shader *p = dynamic_cast<const phong_shader *>(m))
    {
        if (field(*p, ps_rf{}) != 0.0f || field(*p, ps_tran{}) != 0.0f || field(*p, ps_td{}) != 0.0f ||
            field(*p, ps_rfd{}) != 0.0f)
            unsupported("a phong_shader with reflection or refraction");
        put3(out.ka, field(*p, ps_ka{}));
        put3(out.kd, field(*p, ps_kd{}));
        put3(out.ks, field(*p, ps_ks{}));
        out.ns = field(*p, ps_s{});
        out.rf = 0.0f;
        out.tran = 0.0f;
        out.ri = 1.0f;
        out.flags = RT_MAT_NO_VERTEX_COLOUR;
        out.rfd = 0.0f;
        out.td = 0.0f;
        return out;
    }
    unsupported("a material other than coloured_mapper_shader and phong_shader");
    return out;
}

// rt_light of a RAPTor light, following how light::find_rays (light.h:62-100)
// and get_light_intensity (light.h:44-59) treat it with one shadow ray per
// light: n.x == 2 (the spherical and triangle constructors) is a point light
// at the centre; otherwise s_b != 0 is a spot light, s_b == 0 a directional
// light along n.  The colour is taken as stored (already divided by 255).
rt_light describe(const light &l)
{
    rt_light out;
    const point_t<> &n = field(l, light_n{});
    const float s_b = field(l, light_s_b{});
    int32_t kind;
    if (n.x == 2.0f)
        kind = RT_LIGHT_POINT;
    else if (s_b != 0.0f)
        kind = RT_LIGHT_SPOT;
    else
        kind = RT_LIGHT_DIRECTIONAL;
    out.kind = kind | RT_LIGHT_UNIT_RGB;
    put3(out.rgb, field(l, light_rgb{}));
    put3(out.pos, l.get_centre());
    put3(out.dir, n);
    out.d = field(l, light_d{});
    out.s_a = field(l, light_s_a{});
    out.s_b = s_b;
    return out;
}

// rt_camera of the camera's internal (supersampled) grid: x_m = -w,
// x_inc = 2w / x_res (camera.h:55-62), so w = -x_m reproduces the grid.
rt_camera describe(const camera &c)
{
    if (field(c, cam_tm{}) != nullptr) unsupported("a sky box background");
    if (field(c, cam_aperture{}) > 0.0f && field(c, cam_focal_length{}) > 0.0f) unsupported("depth of field");
    rt_camera out;
    put3(out.pos, c.camera_position());
    // with the identity orientation hand over the stored axes: the core
    // applies the identity rotation itself, exactly as base_camera does
    const quaternion_t &q = c.orientation();
    const bool identity = q.w == 1.0f && q.x == 0.0f && q.y == 0.0f && q.z == 0.0f && !std::signbit(q.x) &&
                          !std::signbit(q.y) && !std::signbit(q.z);
    const base_camera &bc = c;
    put3(out.x_axis, identity ? field(bc, bcam_x{}) : c.x_axis());
    put3(out.y_axis, identity ? field(bc, bcam_y{}) : c.y_axis());
    put3(out.z_axis, identity ? field(bc, bcam_z{}) : c.z_axis());
    put3(out.background, field(c, cam_b{}));
    out.w = -field(c, cam_x_m{});
    out.h = -field(c, cam_y_m{});
    out.t = field(c, cam_t{});
    out.xres = (int32_t)field(c, cam_x_res{});
    out.yres = (int32_t)field(c, cam_y_res{});
    return out;
}

void vertices_of(const primitive_store &prims, std::vector<float> &verts)
{
    const int n = prims.size();
    verts.resize(9 * (size_t)n);
    for (int i = 0; i < n; ++i)
    {
        const triangle *t = prims.primitive(i);
        put3(&verts[9 * (size_t)i + 0], t->get_vertex_a());
        put3(&verts[9 * (size_t)i + 3], t->get_vertex_b());
        put3(&verts[9 * (size_t)i + 6], t->get_vertex_c());
    }
}
}  // namespace gpu_detail

using namespace gpu_detail;

gpu_bvh::gpu_bvh(const primitive_store &prims, int device) : _scene(nullptr)
{
    check(rt_scene_create(context(device), &_scene));
    const int n = prims.size();
    std::vector<float> verts;
    vertices_of(prims, verts);
    std::vector<int32_t> idx(3 * (size_t)n);
    std::vector<uint32_t> flags((size_t)n);
    std::vector<int32_t> mat((size_t)n);
    std::vector<float> attr, normals;
    std::map<const material *, int32_t> mat_index;
    for (int i = 0; i < n; ++i)
    {
        const triangle *t = prims.primitive(i);
        for (int k = 0; k < 3; ++k) idx[3 * (size_t)i + k] = 3 * i + k;
        const material *m = material_of(*t);
        auto it = mat_index.find(m);
        if (it == mat_index.end())
        {
            it = mat_index.emplace(m, (int32_t)_materials.size()).first;
            _materials.push_back(m);
        }
        mat[i] = it->second;
        flags[i] = (t->get_light() ? RT_TRI_LIGHT : 0u) | (m && m->is_transparent() ? RT_TRI_TRANSPARENT : 0u);
        // vertex normals vnt[0..2] and attributes vnt[3..5] (triangle.h:124-176),
        // each present unless its first x is MAX_DIST
        const point_t<> *vnt = field(*t, tri_vnt{});
        if (vnt && vnt[3].x != MAX_DIST)
        {
            if (attr.empty()) attr.assign(9 * (size_t)n, 0.0f);
            for (int k = 0; k < 3; ++k) put3(&attr[9 * (size_t)i + 3 * k], vnt[3 + k]);
        }
        if (vnt && vnt[0].x != MAX_DIST)
        {
            if (normals.empty())
            {
                // triangles without vertex normals keep their face normal
                normals.assign(9 * (size_t)n, 0.0f);
                for (int j = 0; j < n; ++j) normals[9 * (size_t)j] = FLT_MAX;
            }
            for (int k = 0; k < 3; ++k) put3(&normals[9 * (size_t)i + 3 * k], vnt[k]);
        }
    }
    if (_materials.size() > RT_MAX_MATERIALS)
        unsupported("more than RT_MAX_MATERIALS distinct materials");
    check(rt_scene_upload(_scene, verts.data(), 3 * n, idx.data(), n, attr.empty() ? nullptr : attr.data(),
                          flags.data()));
    if (_materials.size() > 1) check(rt_scene_set_materials(_scene, mat.data(), n));
    if (!normals.empty()) check(rt_scene_set_normals(_scene, normals.data(), n));
    check(rt_bvh_build(_scene, nullptr));
}

void gpu_bvh::refit(const primitive_store &prims)
{
    std::vector<float> verts;
    vertices_of(prims, verts);
    check(rt_scene_refit_vertices(_scene, verts.data(), 3 * prims.size(), nullptr));
}

int64_t &ray_tracer_gpu_stream_position()
{
    static int64_t pos = 0;
    return pos;
}

uint64_t &ray_tracer_gpu_pixel_seed()
{
    static uint64_t seed = 0;
    return seed;
}

void ray_tracer_gpu(const ssd *const sub_division, const light_list &lights, const primitive_store &everything,
                    camera &c)
{
    const gpu_bvh *accel = dynamic_cast<const gpu_bvh *>(sub_division);
    std::unique_ptr<gpu_bvh> own;
    if (!accel)
    {
        own.reset(new gpu_bvh(everything));
        accel = own.get();
    }
    const rt_camera cam = describe(c);
    if (lights.size() > RT_MAX_LIGHTS) unsupported("more than RT_MAX_LIGHTS lights");
    std::vector<rt_light> ls;
    for (const light &l : lights) ls.push_back(describe(l));
    std::vector<rt_material> mats;
    for (const material *m : accel->materials()) mats.push_back(describe(m));
    const size_t nsamples = (size_t)cam.xres * (size_t)cam.yres;
    std::vector<float> image(3 * nsamples);
    // the compile-time sampling of the build this is compiled into
    // (common.h:34-44): SOFT_SHADOW shadow rays per light, DIFFUSE_REFLECTIONS
    // rays per diffuse reflection
#ifdef SOFT_SHADOW
    const int32_t soft = (int32_t)(SOFT_SHADOW);
#else
    const int32_t soft = 1;
#endif
#ifdef DIFFUSE_REFLECTIONS
    const int32_t diffuse = (int32_t)(DIFFUSE_REFLECTIONS);
#else
    const int32_t diffuse = 0;
#endif
    if (soft > 1 || diffuse > 0)
    {
        // lights' extents: the radius of a spherical light, the triangles of
        // a triangle-defined one (light.h:17-29); a directional light has none
        std::vector<rt_light_shape> shapes(ls.size());
        std::vector<std::vector<int32_t>> tris(ls.size());
        size_t i = 0;
        for (const light &l : lights)
        {
            shapes[i].radius = field(l, light_r{});
            shapes[i].ntris = 0;
            shapes[i].tris = nullptr;
            const std::vector<int> *t = field(l, light_t{});
            if (t && !t->empty() && (ls[i].kind & 0xff) != RT_LIGHT_DIRECTIONAL)
            {
                tris[i].assign(t->begin(), t->end());
                shapes[i].ntris = (int32_t)tris[i].size();
                shapes[i].tris = tris[i].data();
            }
            ++i;
        }
        bool spread = false;
        for (const rt_material &m : mats)
            spread = spread || (diffuse > 0 && ((m.rf > 0.0f && m.rfd != 0.0f) || (m.tran > 0.0f && m.td != 0.0f)));
        rt_sampling smp;
        smp.soft_samples = soft;
        smp.diffuse_samples = diffuse;
        smp.stream = spread ? RT_STREAM_PIXEL : RT_STREAM_REFERENCE;
        smp.reserved = 0;
        smp.stream_offset = ray_tracer_gpu_stream_position();
        smp.seed = ray_tracer_gpu_pixel_seed();
        int64_t end = 0;
        check(rt_render_distributed(accel->scene(), &cam, ls.data(), (int32_t)ls.size(), shapes.data(), mats.data(),
                                    (int32_t)mats.size(), &smp, nullptr, image.data(), &end, nullptr));
        if (spread) ++ray_tracer_gpu_pixel_seed();
        else ray_tracer_gpu_stream_position() = end;
    }
    else
    {
        check(rt_render_image(accel->scene(), &cam, ls.data(), (int32_t)ls.size(), mats.data(), (int32_t)mats.size(),
                              image.data(), nullptr));
    }
    // camera::set_pixel for every ray of the grid, as ray_trace_one_pixel does
    for (int32_t y = 0; y < cam.yres; ++y)
        for (int32_t x = 0; x < cam.xres; ++x)
        {
            const float *p = &image[3 * ((size_t)x + (size_t)y * (size_t)cam.xres)];
            c.set_pixel(ext_colour_t(p[0], p[1], p[2]), x, y);
        }
}
}  // namespace raptor_raytracer
