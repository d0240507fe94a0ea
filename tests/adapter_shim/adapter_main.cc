// adapter_main.cc -- TEST INFRASTRUCTURE ONLY.  Drives the drop-in adapter
// (raptor_gpu_bvh.h / .cc) the way a RAPTor program drives bvh and
// ray_tracer: builds a primitive_store, lights, materials and a camera from
// the scene file tests/test_gpu_adapter.py writes, calls ray_tracer_gpu and
// camera::clip_image_to_rgb, and answers ray queries through the ssd
// interface.  Usage: adapter_main <scene file> <output file>.
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

#include "raptor_gpu_bvh.h"

using namespace raptor_raytracer;

namespace
{
struct Reader
{
    FILE *f;
    template <typename T>
    std::vector<T> take(size_t n)
    {
        std::vector<T> v(n);
        if (n && fread(v.data(), sizeof(T), n, f) != n) throw std::runtime_error("short scene file");
        return v;
    }
};

// A kd texture mapper of coloured_mapper_shader: marks the material as
// coloured by the triangle's per-vertex attribute.
struct vertex_colour_mapper : texture_mapper
{
};

// An ssd that is not a gpu_bvh: ray_tracer_gpu must build its own.
struct other_ssd : ssd
{
    int find_nearest_object(const ray *const, hit_description *const) const override { return -1; }
    bool found_nearer_object(const ray *const, const float) const override { return false; }
};
}  // namespace

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    FILE *in = fopen(argv[1], "rb");
    if (!in) return 3;
    Reader rd{in};
    const std::vector<int32_t> hdr = rd.take<int32_t>(8);
    const int ntris = hdr[0], nmats = hdr[1], nlights = hdr[2], out_x = hdr[3], out_y = hdr[4], aa_x = hdr[5],
              aa_y = hdr[6], nrays = hdr[7];
    const std::vector<float> cam = rd.take<float>(18);
    const std::vector<float> tris = rd.take<float>(9 * (size_t)ntris);
    const int has_attr = rd.take<int32_t>(1)[0];
    const std::vector<float> attr = rd.take<float>(has_attr ? 9 * (size_t)ntris : 0);
    const int has_normals = rd.take<int32_t>(1)[0];
    const std::vector<float> normals = rd.take<float>(has_normals ? 9 * (size_t)ntris : 0);
    const std::vector<int32_t> mat_idx = rd.take<int32_t>(ntris);
    const std::vector<int32_t> tri_light = rd.take<int32_t>(ntris);
    const std::vector<float> mdesc = rd.take<float>(16 * (size_t)nmats);
    const std::vector<float> ldesc = rd.take<float>(16 * (size_t)nlights);
    const std::vector<float> rays = rd.take<float>(7 * (size_t)nrays);
    const int nlt = rd.take<int32_t>(1)[0];
    const std::vector<int32_t> light_tris = rd.take<int32_t>((size_t)nlt);
    fclose(in);

    vertex_colour_mapper mapper;
    std::vector<std::unique_ptr<material>> mats;
    for (int i = 0; i < nmats; ++i)
    {
        const float *m = &mdesc[16 * (size_t)i];
        const ext_colour_t ka(m[1], m[2], m[3]), kd(m[4], m[5], m[6]), ks(m[7], m[8], m[9]);
        if (m[0] == 0.0f)
            mats.emplace_back(new coloured_mapper_shader(ka, kd, ks, m[10], m[11], m[12], m[13], 0.0f, m[15], nullptr,
                                                         m[14] != 0.0f ? &mapper : nullptr));
        else
            mats.emplace_back(new phong_shader(ka, kd, ks, m[10]));
    }
    primitive_store store;
    for (int i = 0; i < ntris; ++i)
    {
        const float *t = &tris[9 * (size_t)i];
        point_t<> vt[3], vn[3];
        for (int k = 0; k < 3; ++k)
        {
            if (has_attr) vt[k] = point_t<>(attr[9 * (size_t)i + 3 * k], attr[9 * (size_t)i + 3 * k + 1], attr[9 * (size_t)i + 3 * k + 2]);
            if (has_normals) vn[k] = point_t<>(normals[9 * (size_t)i + 3 * k], normals[9 * (size_t)i + 3 * k + 1], normals[9 * (size_t)i + 3 * k + 2]);
        }
        store.emplace_back(mats[mat_idx[i]].get(), point_t<>(t[0], t[1], t[2]), point_t<>(t[3], t[4], t[5]),
                           point_t<>(t[6], t[7], t[8]), tri_light[i] != 0, has_normals ? vn : nullptr,
                           has_attr ? vt : nullptr);
    }
    // kind 0 spherical (radius l[13]), 1 directional, 2 spot (radius l[13]),
    // 3 defined by l[14] triangles of the store (the next ones of light_tris)
    light_list lights;
    std::vector<std::vector<int>> tri_lists;
    tri_lists.reserve((size_t)nlights);
    size_t lt = 0;
    for (int i = 0; i < nlights; ++i)
    {
        const float *l = &ldesc[16 * (size_t)i];
        const ext_colour_t rgb(l[1], l[2], l[3]);
        const point_t<> pos(l[4], l[5], l[6]), dir(l[7], l[8], l[9]);
        if (l[0] == 0.0f) lights.emplace_back(rgb, pos, l[10], l[13]);
        else if (l[0] == 1.0f) lights.emplace_back(rgb, dir, l[10]);
        else if (l[0] == 2.0f) lights.emplace_back(rgb, pos, dir, l[10], l[11], l[12], l[13]);
        else
        {
            const size_t k = (size_t)l[14];
            if (lt + k > light_tris.size()) return 6;
            tri_lists.emplace_back(light_tris.begin() + (long)lt, light_tris.begin() + (long)(lt + k));
            lt += k;
            lights.emplace_back(&store, rgb, pos, l[10], &tri_lists.back());
        }
    }
    camera c(point_t<>(cam[0], cam[1], cam[2]), point_t<>(cam[3], cam[4], cam[5]), point_t<>(cam[6], cam[7], cam[8]),
             point_t<>(cam[9], cam[10], cam[11]), ext_colour_t(cam[12], cam[13], cam[14]), cam[15], cam[16], cam[17],
             out_x, out_y, aa_x, aa_y, 0.0f, 0.0f);

    FILE *out = fopen(argv[2], "wb");
    if (!out) return 4;
    std::vector<unsigned char> rgb(3 * (size_t)out_x * out_y);
    try
    {
        gpu_bvh accel(store);
        // the drop-in, with the gpu_bvh as the sub-division
        ray_tracer_gpu(&accel, lights, store, c);
        c.clip_image_to_rgb(rgb.data());
        fwrite(rgb.data(), 1, rgb.size(), out);
        // and with another ssd: the adapter builds its own gpu_bvh
        other_ssd other;
        camera c2(point_t<>(cam[0], cam[1], cam[2]), point_t<>(cam[3], cam[4], cam[5]), point_t<>(cam[6], cam[7], cam[8]),
                  point_t<>(cam[9], cam[10], cam[11]), ext_colour_t(cam[12], cam[13], cam[14]), cam[15], cam[16],
                  cam[17], out_x, out_y, aa_x, aa_y, 0.0f, 0.0f);
        ray_tracer_gpu(&other, lights, store, c2);
        c2.clip_image_to_rgb(rgb.data());
        fwrite(rgb.data(), 1, rgb.size(), out);
        // ssd queries: one ray per call, then the batched forms
        std::vector<ray> rs;
        std::vector<float> tm((size_t)nrays);
        for (int i = 0; i < nrays; ++i)
        {
            const float *r = &rays[7 * (size_t)i];
            rs.emplace_back(point_t<>(r[0], r[1], r[2]), r[3], r[4], r[5]);
            tm[i] = r[6];
        }
        std::vector<int32_t> ids((size_t)nrays), ids_b((size_t)nrays);
        std::vector<float> t((size_t)nrays), t_b((size_t)nrays);
        std::vector<uint8_t> occ((size_t)nrays), occ_b((size_t)nrays);
        const ssd *s = &accel;
        for (int i = 0; i < nrays; ++i)
        {
            hit_description h;
            ids[i] = s->find_nearest_object(&rs[i], &h);
            t[i] = h.d;
            occ[i] = s->found_nearer_object(&rs[i], tm[i]) ? 1 : 0;
        }
        std::vector<hit_description> hb((size_t)nrays);
        std::unique_ptr<bool[]> ob(new bool[(size_t)nrays + 1]);
        accel.find_nearest_objects(rs.data(), nrays, ids_b.data(), hb.data());
        accel.found_nearer_objects(rs.data(), tm.data(), nrays, ob.get());
        for (int i = 0; i < nrays; ++i)
        {
            t_b[i] = hb[i].d;
            occ_b[i] = ob[i] ? 1 : 0;
        }
        fwrite(ids.data(), 4, ids.size(), out);
        fwrite(t.data(), 4, t.size(), out);
        fwrite(occ.data(), 1, occ.size(), out);
        fwrite(ids_b.data(), 4, ids_b.size(), out);
        fwrite(t_b.data(), 4, t_b.size(), out);
        fwrite(occ_b.data(), 1, occ_b.size(), out);
    }
    catch (const std::exception &e)
    {
        fprintf(stderr, "%s\n", e.what());
        fclose(out);
        return 5;
    }
    fclose(out);
    return 0;
}
