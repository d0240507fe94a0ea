"""The C++ drop-in adapter (raptor_gb300/host/raptor_gpu_bvh.h) compiles
against the reference's own headers: gpu_bvh is a raptor_raytracer::ssd and
ray_tracer_gpu takes the reference's camera.  Runs only where the reference
tree is present (compile-only; nothing is executed)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("RAPTOR_REF", "/root/reference/RAPTor")

TU = r'''
#include "raptor_gpu_bvh.h"
using namespace raptor_raytracer;
int use(primitive_store &s, camera &c) {
    gpu_bvh b(s);
    const ssd *as_ssd = &b;
    ray r(point_t<>(0, 0, 0), 0.f, 0.f, 1.f);
    hit_description h;
    const int id = as_ssd->find_nearest_object(&r, &h);
    const bool o = as_ssd->found_nearer_object(&r, 1.0f);
    gpu_camera_args ca{};
    std::vector<gpu_light_args> ls(1);
    ray_tracer_gpu(&b, ls, ca, c, ext_colour_t(0, 0, 0), ext_colour_t(1, 1, 1), ext_colour_t(1, 1, 1), 10.f);
    return id + (o ? 1 : 0);
}
'''


@pytest.mark.skipif(not os.path.isdir(REF) or shutil.which("g++") is None, reason="reference tree not present")
def test_adapter_compiles_against_reference_headers(tmp_path):
    tu = tmp_path / "tu.cc"
    tu.write_text(TU)
    inc = ["common", "raytracer", "raytracer/spatial_sub_division", "raytracer/materials", "raytracer/parsers",
           "parsers", "sdl_wrappers"]
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-include", "memory", "-include", "cstdint", "-include",
           "algorithm", "-DREFLECTIONS_ON", "-DREFRACTIONS_ON", "-DEXACT_NORMALISE",
           "-I", os.path.join(ROOT, "oracle", "refbuild", "shim")]
    cmd += sum((["-I", os.path.join(REF, d)] for d in inc), [])
    cmd += ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "raptor_gb300", "host")]
    if os.uname().machine in ("x86_64", "AMD64"):
        cmd.append("-msse4.1")
    cmd.append(str(tu))
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
