"""The C++ drop-in adapter (raptor_gb300/host/raptor_gpu_bvh.{h,cc})
compiles against the reference's own headers: gpu_bvh is a
raptor_raytracer::ssd and ray_tracer_gpu has ray_tracer's signature
(raytracer.h:105), reading the private fields it needs from the real
classes.  Runs only where the reference tree is present (compiled, not run:
the reference's headers are x86-only; tests/test_gpu_adapter.py runs the
adapter on the GPU against stand-ins of those headers)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("RAPTOR_REF", "/root/reference/RAPTor")

TU = r'''
#include "raptor_gpu_bvh.h"
#include "raytracer.h"
using namespace raptor_raytracer;
int use(primitive_store &s, const light_list &lights, camera &c) {
    gpu_bvh b(s);
    const ssd *as_ssd = &b;
    ray r(point_t<>(0, 0, 0), 0.f, 0.f, 1.f);
    hit_description h;
    const int id = as_ssd->find_nearest_object(&r, &h);
    const bool o = as_ssd->found_nearer_object(&r, 1.0f);
    // the drop-in has ray_tracer's exact type
    void (*reference)(const ssd *const, const light_list &, const primitive_store &, camera &) = &ray_tracer;
    void (*gpu)(const ssd *const, const light_list &, const primitive_store &, camera &) = &ray_tracer_gpu;
    (void)reference;
    gpu(as_ssd, lights, s, c);
    return id + (o ? 1 : 0);
}
'''


def compile_cmd(out_flag, src, tmp_path):
    inc = ["common", "raytracer", "raytracer/spatial_sub_division", "raytracer/materials", "raytracer/parsers",
           "parsers", "sdl_wrappers"]
    cmd = ["g++", "-std=c++17", out_flag, "-w", "-include", "memory", "-include", "cstdint", "-include",
           "algorithm", "-DREFLECTIONS_ON", "-DREFRACTIONS_ON", "-DEXACT_NORMALISE",
           "-I", os.path.join(ROOT, "oracle", "refbuild", "shim")]
    cmd += sum((["-I", os.path.join(REF, d)] for d in inc), [])
    cmd += ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "raptor_gb300", "host")]
    if os.uname().machine in ("x86_64", "AMD64"):
        cmd.append("-msse4.1")
    cmd.append(str(src))
    if out_flag == "-c":
        cmd += ["-o", str(tmp_path / "adapter.o")]
    return cmd


@pytest.mark.skipif(not os.path.isdir(REF) or shutil.which("g++") is None, reason="reference tree not present")
def test_adapter_compiles_against_reference_headers(tmp_path):
    tu = tmp_path / "tu.cc"
    tu.write_text(TU)
    r = subprocess.run(compile_cmd("-fsyntax-only", tu, tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # the adapter's source, with its reads of the reference's private fields
    src = os.path.join(ROOT, "raptor_gb300", "host", "raptor_gpu_bvh.cc")
    r = subprocess.run(compile_cmd("-c", src, tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(not os.path.isdir(REF) or shutil.which("g++") is None, reason="reference tree not present")
def test_adapter_compiles_into_soft_shadow_builds(tmp_path):
    """raptor_gpu_bvh.cc compiled as a SOFT_SHADOW / DIFFUSE_REFLECTIONS
    build of the reference compiles it, reading the lights' radius and
    triangle list (light.h:228-233) for rt_render_distributed."""
    src = os.path.join(ROOT, "raptor_gb300", "host", "raptor_gpu_bvh.cc")
    for defines in (["-DSOFT_SHADOW=16"], ["-DSOFT_SHADOW=16", "-DDIFFUSE_REFLECTIONS=16"]):
        cmd = compile_cmd("-c", src, tmp_path)
        cmd[2:2] = defines
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, (defines, r.stderr[-3000:])
