// raptor_stand_in.h -- TEST INFRASTRUCTURE ONLY.  Minimal stand-ins for the
// RAPTor classes the drop-in adapter (raptor_gb300/host/raptor_gpu_bvh.*)
// touches, with the reference's names, member names, member types and
// constructor arguments, so the adapter can be compiled and run where the
// reference tree cannot (its common/simd.h is x86-only).  Only the parts the
// adapter and its test use exist; tests/test_host_adapter.py compiles the
// adapter against the reference's real headers.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector>

const float MAX_DIST = FLT_MAX;   // common/common.h

template <class T = float>
class point_t
{
    public :
        T x, y, z;
        point_t(const T x = 0.0f, const T y = 0.0f, const T z = 0.0f) : x(x), y(y), z(z) {}
};

// quaternion_t (common/quaternion_t.h): public w, x, y, z; rotate() is the
// identity for the identity orientation, the only one the stand-in needs.
class quaternion_t
{
    public :
        quaternion_t() : w(1.0f), x(0.0f), y(0.0f), z(0.0f) {}
        point_t<> rotate(const point_t<> &p) const { return p; }
        float w, x, y, z;
};

class base_camera
{
    public :
        base_camera(const point_t<> &c, const point_t<> &x, const point_t<> &y, const point_t<> &z, const float speed)
            : _c(c), _x(x), _y(y), _z(z), _speed(speed) {}
        virtual ~base_camera() {}
        const point_t<> &camera_position() const { return _c; }
        const quaternion_t &orientation() const { return _o; }
        point_t<> x_axis() const { return _o.rotate(_x); }
        point_t<> y_axis() const { return _o.rotate(_y); }
        point_t<> z_axis() const { return _o.rotate(_z); }
    private :
        point_t<> _c;
        quaternion_t _o;
        point_t<> _x;
        point_t<> _y;
        point_t<> _z;
        float _speed;
};

namespace raptor_raytracer
{
class ext_colour_t
{
    public :
        float r, g, b;
        ext_colour_t(const float r, const float g, const float b) : r(r), g(g), b(b) {}
        ext_colour_t(const float r = 0.0f) : r(r), g(r), b(r) {}
};

enum class hit_t : char { miss = 0, out_in = 1, in_out = 2 };

class hit_description
{
    public :
        hit_description(const float d = MAX_DIST, const hit_t h = hit_t::miss, const float u = 0.0f, const float v = 0.0f)
            : u(u), v(v), d(d), h(h) {}
        float u, v, d;
        hit_t h;
};

class ray
{
    public :
        ray(const point_t<> &o, const float x = 0.0f, const float y = 0.0f, const float z = 0.0f)
            : ogn(o), dir(x, y, z) {}
        point_t<> get_ogn() const { return ogn; }
        point_t<> get_dir() const { return dir; }
    private :
        point_t<> ogn, dir;
};

class texture_mapper
{
    public :
        virtual ~texture_mapper() {}
};

class material
{
    public :
        material(const bool t = false) : t(t) {}
        virtual ~material() {}
        bool is_transparent() const { return t; }
    private :
        const bool t;
};

class coloured_mapper_shader : public material
{
    public :
        coloured_mapper_shader(const ext_colour_t &ka, const ext_colour_t &kd, const ext_colour_t &ks = 0.0f,
                               const float ns = 0.0f, const float tran = 0.0f, const float ri = 1.0f,
                               const float rf = 0.0f, const float td = 0.0f, const float rfd = 0.0f,
                               const texture_mapper *const t_ka = nullptr, const texture_mapper *const t_kd = nullptr)
            : material(tran > 0.0f), t_ka(t_ka), t_kd(t_kd), t_ks(nullptr), t_ns(nullptr), t_refl(nullptr),
              t_d(nullptr), ka(ka), kd(kd), ks(ks), ns(ns), tran(tran), ri(ri), rf(rf), td(td), rfd(rfd) {}
    private :
        const texture_mapper *t_ka;
        const texture_mapper *t_kd;
        const texture_mapper *t_ks;
        const texture_mapper *t_ns;
        const texture_mapper *t_refl;
        const texture_mapper *t_d;
        const ext_colour_t ka;
        const ext_colour_t kd;
        const ext_colour_t ks;
        const float ns;
        const float tran;
        const float ri;
        const float rf;
        const float td;
        const float rfd;
};

class phong_shader : public material
{
    public :
        phong_shader(const ext_colour_t &ka, const ext_colour_t &kd, const ext_colour_t &ks, const float s = 0.0f,
                     const float tran = 0.0f, const float ri = 1.0f, const float rf = 0.0f, const float td = 0.0f,
                     const float rfd = 0.0f)
            : material(tran > 0.0f), ka(ka), kd(kd), ks(ks), s(s), tran(tran), ri(ri), rf(rf), td(td), rfd(rfd) {}
    private :
        const ext_colour_t ka;
        const ext_colour_t kd;
        const ext_colour_t ks;
        const float s;
        const float tran;
        const float ri;
        const float rf;
        const float td;
        const float rfd;
};

// triangle (triangle.h:20-176): material pointer with the light flag in
// bit 0, optional vertex normals vnt[0..2] and attributes vnt[3..5].
class triangle
{
    public :
        triangle(material *const m, const point_t<> &a, const point_t<> &b, const point_t<> &c, bool l = false,
                 const point_t<> *v_n = nullptr, const point_t<> *v_t = nullptr)
            : m(reinterpret_cast<std::int64_t>(m) | (l ? 1 : 0)), vnt(nullptr), vertex_a(a), vertex_b(b), vertex_c(c)
        {
            if (v_n || v_t)
            {
                vnt = new point_t<>[6];
                if (v_n) { vnt[0] = v_n[0]; vnt[1] = v_n[1]; vnt[2] = v_n[2]; }
                else vnt[0].x = MAX_DIST;
                if (v_t) { vnt[3] = v_t[0]; vnt[4] = v_t[1]; vnt[5] = v_t[2]; }
                else vnt[3].x = MAX_DIST;
            }
        }
        triangle(triangle &&r) : m(r.m), vnt(r.vnt), vertex_a(r.vertex_a), vertex_b(r.vertex_b), vertex_c(r.vertex_c)
        {
            r.vnt = nullptr;
        }
        ~triangle() { delete[] vnt; }
        bool get_light() const { return m & 0x1; }
        point_t<> get_vertex_a() const { return vertex_a; }
        point_t<> get_vertex_b() const { return vertex_b; }
        point_t<> get_vertex_c() const { return vertex_c; }
    private :
        std::int64_t m;
        point_t<> *vnt;
        point_t<> vertex_a;
        point_t<> vertex_b;
        point_t<> vertex_c;
};

class primitive_store
{
    public :
        template <class... Args>
        int emplace_back(Args... args)
        {
            _prims.emplace_back(args...);
            return (int)_prims.size() - 1;
        }
        triangle *primitive(const int i) { return &_prims[i]; }
        const triangle *primitive(const int i) const { return &_prims[i]; }
        int size() const { return (int)_prims.size(); }
    private :
        std::vector<triangle> _prims;
};

class ssd
{
    public :
        virtual ~ssd() {}
        virtual int find_nearest_object(const ray *const r, hit_description *const h) const = 0;
        virtual bool found_nearer_object(const ray *const r, const float t) const = 0;
};

// light (light.h:14-213): rgb stored divided by 255; n = (2, 2, 2) marks the
// spherical (point) light.
class light
{
    public :
        light(const ext_colour_t &rgb, const point_t<> &c, const float d, const float r)
            : e(nullptr), t(nullptr), rgb(rgb.r / 255.0f, rgb.g / 255.0f, rgb.b / 255.0f), c(c), n(2.0f, 2.0f, 2.0f),
              r(r), d(d), s_a(0.0f), s_b(0.0f) {}
        light(const ext_colour_t &rgb, const point_t<> &c, const point_t<> &n, const float d, const float s_a,
              const float s_b, const float r)
            : e(nullptr), t(nullptr), rgb(rgb.r / 255.0f, rgb.g / 255.0f, rgb.b / 255.0f), c(c), n(n), r(r), d(d),
              s_a(s_a), s_b(s_b) {}
        light(const ext_colour_t &rgb, const point_t<> &n, const float d)
            : e(nullptr), t(nullptr), rgb(rgb.r / 255.0f, rgb.g / 255.0f, rgb.b / 255.0f), c(), n(n), r(0.0f), d(d),
              s_a(0.0f), s_b(0.0f) {}
        light(const primitive_store *const e, const ext_colour_t &rgb, const point_t<> &c, const float d,
              const std::vector<int> *const t)
            : e(e), t(t), rgb(rgb.r / 255.0f, rgb.g / 255.0f, rgb.b / 255.0f), c(c), n(2.0f, 2.0f, 2.0f), r(0.0f),
              d(d), s_a(0.0f), s_b(0.0f) {}
        const point_t<> &get_centre() const { return c; }
    private :
        const primitive_store *const e;
        const std::vector<int> *const t;
        const ext_colour_t rgb;
        const point_t<> c;
        const point_t<> n;
        const float r;
        const float d;
        const float s_a;
        const float s_b;
};

typedef std::vector<light> light_list;

// camera (camera.h:52-555): the pinhole constructor, set_pixel and
// clip_image_to_rgb (camera.h:281-319).
class camera : public base_camera
{
    public :
        camera(const point_t<> &c, const point_t<> &x, const point_t<> &y, const point_t<> &z, const ext_colour_t &b,
               const float w, const float h, const float t, const unsigned x_res, const unsigned y_res,
               const unsigned x_a_res, const unsigned y_a_res, const float aperture, const float focal_length)
            : base_camera(c, x, y, z, 1.0f), tm(nullptr), image(new ext_colour_t[(x_res * x_a_res) * (y_res * y_a_res)]),
              b(b), x_m(-w), y_m(-h), x_inc((w * 2.0f) / static_cast<float>(x_res * x_a_res)),
              y_inc((h * 2.0f) / static_cast<float>(y_res * y_a_res)), t(t), x_res(x_res * x_a_res),
              y_res(y_res * y_a_res), out_x_res(x_res), out_y_res(y_res), aperture(aperture),
              focal_length(focal_length) {}
        ~camera() { delete[] image; }
        camera &set_pixel(const ext_colour_t &p, const int x, const int y)
        {
            image[x + (y * x_res)] = p;
            return *this;
        }
        void clip_image_to_rgb(unsigned char *c) const
        {
            const int xs = (int)(x_res / out_x_res), ys = (int)(y_res / out_y_res), n = xs * ys;
            for (int x = 0; x < (int)out_x_res; ++x)
                for (int y = 0; y < (int)out_y_res; ++y)
                {
                    ext_colour_t a(0.0f, 0.0f, 0.0f);
                    const int base = (x * xs) + (y * ys * (int)x_res);
                    for (int a_x = 0; a_x < xs; ++a_x)
                        for (int a_y = 0; a_y < ys; ++a_y)
                        {
                            a.r += image[base + (a_y * x_res) + a_x].r;
                            a.g += image[base + (a_y * x_res) + a_x].g;
                            a.b += image[base + (a_y * x_res) + a_x].b;
                        }
                    const int o = (x + (y * (int)out_x_res)) * 3;
                    c[o] = (unsigned char)std::fmin(255.0f, std::fmax(0.0f, a.r / n));
                    c[o + 1] = (unsigned char)std::fmin(255.0f, std::fmax(0.0f, a.g / n));
                    c[o + 2] = (unsigned char)std::fmin(255.0f, std::fmax(0.0f, a.b / n));
                }
        }
        unsigned x_resolution() const { return out_x_res; }
        unsigned y_resolution() const { return out_y_res; }
    private :
        const std::vector<texture_mapper *> *const tm;
        ext_colour_t *image;
        const ext_colour_t b;
        const float x_m;
        const float y_m;
        const float x_inc;
        const float y_inc;
        const float t;
        const unsigned x_res;
        const unsigned y_res;
        const unsigned out_x_res;
        const unsigned out_y_res;
        float aperture;
        float focal_length;
};
}  // namespace raptor_raytracer
