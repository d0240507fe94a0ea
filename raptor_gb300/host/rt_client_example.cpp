// rt_client_example.cpp -- a plain C++ client of the C ABI (include/rtcore.h),
// the way RAPTor's own C++ would call it: build the 6-triangle x-axis
// fixture of raytracer/unit_tests/bih_tests.cc:31-38, ask the questions of
// that file's x_ray_* cases through rt_trace_closest / rt_trace_any, and
// check the answers.  Exits 0 when every answer matches.
#include <cmath>
#include <cstdio>
#include <vector>

#include "rtcore.h"

namespace {

struct Case {
    const char *name;
    float o[3], d[3];
    int nearest;        // -2: not asked
    float distance;     // < 0: not asked
    float nearer_t;     // < 0: not asked
    int nearer;
};

int fail(const char *what)
{
    std::fprintf(stderr, "%s: %s\n", what, rt_last_error_string());
    return 1;
}

}  // namespace

int main()
{
    // x_tris of the bih test fixture: two 9x9 squares at x=0, 2x2 at x=1, 2x2 at x=10
    const float tri[6][3][3] = {
        {{0, 0, 0}, {0, 9, 0}, {0, 9, 9}}, {{0, 0, 0}, {0, 9, 9}, {0, 0, 9}},
        {{1, 0, 0}, {1, 2, 0}, {1, 2, 2}}, {{1, 0, 0}, {1, 2, 2}, {1, 0, 2}},
        {{10, 3, 0}, {10, 5, 0}, {10, 5, 2}}, {{10, 3, 0}, {10, 5, 2}, {10, 3, 2}},
    };
    std::vector<float> verts;
    std::vector<int32_t> idx;
    for (int t = 0; t < 6; ++t)
        for (int k = 0; k < 3; ++k) {
            for (int c = 0; c < 3; ++c) verts.push_back(tri[t][k][c]);
            idx.push_back(3 * t + k);
        }
    const Case cases[] = {
        {"x_ray_miss_world", {15.f, 9.1f, 0.f}, {-1.f, 0.f, 0.f}, -1, -1.f, 1.f, 0},
        {"x_ray_away_from_world", {20.f, 5.f, 0.f}, {1.f, 0.f, 0.f}, -1, -1.f, 1.f, 0},
        {"x_ray_pass_between", {5.f, 5.f, -10.f}, {0.f, 0.f, 1.f}, -1, -1.f, 100.f, 0},
        {"x_ray_stuck_in_middle", {5.f, 5.f, 0.f}, {1.f, 0.f, 0.f}, -2, -1.f, 1.f, 0},
        {"x_ray_hit_in_near", {15.f, 4.f, 0.1f}, {-1.f, 0.f, 0.f}, 4, 5.f, 5.1f, 1},
        {"x_ray_hit_in_near_reverse", {-15.f, 4.f, 0.1f}, {1.f, 0.f, 0.f}, 0, 15.f, 15.1f, 1},
        {"x_ray_hit_in_far", {15.f, 8.f, 0.1f}, {-1.f, 0.f, 0.f}, 0, 15.f, 15.1f, 1},
    };
    rt_context *ctx = nullptr;
    rt_scene *scene = nullptr;
    if (rt_ctx_create(0, &ctx) != RT_OK) return fail("rt_ctx_create");
    if (rt_scene_create(ctx, &scene) != RT_OK) return fail("rt_scene_create");
    if (rt_scene_upload(scene, verts.data(), 18, idx.data(), 6, nullptr, nullptr) != RT_OK) return fail("upload");
    if (rt_bvh_build(scene, nullptr) != RT_OK) return fail("build");
    int bad = 0;
    for (const Case &c : cases) {
        rt_ray r = {c.o[0], c.o[1], c.o[2], c.nearer_t, c.d[0], c.d[1], c.d[2], 0.f};
        rt_hit h;
        uint8_t occ = 0;
        if (rt_trace_closest(scene, &r, 1, &h) != RT_OK) return fail("trace_closest");
        if (rt_trace_any(scene, &r, 1, &occ) != RT_OK) return fail("trace_any");
        bool ok = true;
        if (c.nearest != -2 && h.tri != c.nearest) ok = false;
        if (c.distance >= 0.f && std::fabs(h.t - c.distance) > c.distance * 1e-7f) ok = false;
        if (c.nearer_t >= 0.f && (int)occ != c.nearer) ok = false;
        std::printf("%-28s tri %2d t %-10g occluded %d  %s\n", c.name, h.tri, (double)h.t, occ, ok ? "ok" : "WRONG");
        bad += ok ? 0 : 1;
    }
    rt_scene_destroy(scene);
    rt_ctx_destroy(ctx);
    return bad == 0 ? 0 : 2;
}
