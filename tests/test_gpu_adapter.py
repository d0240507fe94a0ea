"""The C++ drop-in adapter run on the GPU: a program written against RAPTor's
API (tests/adapter_shim/adapter_main.cc, compiled with stand-ins of the
reference's headers, which cannot be compiled on every host) builds a
primitive_store, lights, materials and a camera, calls
ray_tracer_gpu(ssd*, light_list&, primitive_store&, camera&) -- ray_tracer's
signature -- and camera::clip_image_to_rgb, and queries the gpu_bvh through
the ssd interface.  Its frames must equal the C ABI's own renders of the
same scene bit for bit (and so the oracle's within the parity criteria), for
the sub-division being the gpu_bvh or any other ssd, with anti-aliasing,
material tables, mirror materials, directional and spot lights and vertex
normals; its ray queries must equal rt_trace_closest / rt_trace_any."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from parity import PIX_FRAC, pixel_agreement

pytestmark = pytest.mark.gpu

NO_VERTEX_COLOUR = 1


def compile_adapter(tmp_path_factory, defines=()):
    """adapter_main + raptor_gpu_bvh.cc against the stand-in headers, with
    the build's defines (e.g. SOFT_SHADOW=16, as a RAPTor build sets it)."""
    from raptor_gb300 import build
    exe = tmp_path_factory.mktemp("adapter") / "adapter_main"
    shim = os.path.join(ROOT, "tests", "adapter_shim")
    cmd = ["g++", "-std=c++17", "-O2", *[f"-D{d}" for d in defines], "-I", shim, "-I",
           os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "raptor_gb300", "host"),
           os.path.join(shim, "adapter_main.cc"), os.path.join(ROOT, "raptor_gb300", "host", "raptor_gpu_bvh.cc"),
           "-L", build.OUT_DIR, "-lrtcore", f"-Wl,-rpath,{build.OUT_DIR}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.fixture(scope="module")
def adapter_exe(rtlib, tmp_path_factory):
    return compile_adapter(tmp_path_factory)


def run_adapter(exe, tmp_path, scene, frame, materials, mat_of_tri, aa, rays, tmax, kinds):
    """Writes the scene file adapter_main reads, runs it, returns its two
    RGB8 frames and the single-ray and batched query answers.  kinds:
    per material 0 (coloured_mapper_shader) or 1 (phong_shader)."""
    V, T = scene["verts"], scene["tris"]
    nt = T.shape[0]
    cam = frame["camera"]
    lights = frame["lights"]
    W, H = cam["xres"], cam["yres"]
    hdr = np.array([nt, len(materials), len(lights), W, H, aa[0], aa[1], rays.shape[0]], np.int32)
    camv = np.array([*cam["pos"], *cam["x_axis"], *cam["y_axis"], *cam["z_axis"], *cam["background"], cam["w"],
                     cam["h"], cam["t"]], np.float32)
    tris = V[T].reshape(nt, 9).astype(np.float32)
    attr = scene.get("vattr")
    normals = scene.get("corner_normals")
    mats = np.zeros((len(materials), 16), np.float32)
    for i, (m, k) in enumerate(zip(materials, kinds)):
        mats[i, 0] = k
        mats[i, 1:4], mats[i, 4:7], mats[i, 7:10] = m["ka"], m["kd"], m["ks"]
        mats[i, 10:14] = [m["ns"], m.get("tran", 0.0), m.get("ri", 1.0), m.get("rf", 0.0)]
        mats[i, 14] = 0.0 if m.get("flags", 0) & NO_VERTEX_COLOUR else 1.0
        mats[i, 15] = m.get("rfd", 0.0)
    ls = np.zeros((len(lights), 16), np.float32)
    light_tris = []
    for i, l in enumerate(lights):
        ls[i, 0] = 3 if l.get("tris") is not None else l["kind"]
        ls[i, 1:4], ls[i, 4:7], ls[i, 7:10] = l["rgb"], l["pos"], l["dir"]
        ls[i, 10:14] = [l["d"], l.get("s_a", 0.0), l.get("s_b", 0.0), l.get("r", 0.0)]
        if l.get("tris") is not None:
            ls[i, 14] = len(l["tris"])
            light_tris.extend(l["tris"])
    flags = scene.get("flags")
    light_tri = np.zeros(nt, np.int32) if flags is None else (np.asarray(flags) & 1).astype(np.int32)
    path = tmp_path / "scene.bin"
    with open(path, "wb") as f:
        for a in (hdr, camv, tris):
            f.write(a.tobytes())
        f.write(np.int32(attr is not None).tobytes())
        if attr is not None:
            f.write(np.asarray(attr, np.float32)[T].reshape(nt, 9).tobytes())
        f.write(np.int32(normals is not None).tobytes())
        if normals is not None:
            f.write(np.asarray(normals, np.float32).reshape(nt, 9).tobytes())
        for a in (np.asarray(mat_of_tri, np.int32), light_tri, mats, ls):
            f.write(a.tobytes())
        f.write(np.concatenate([rays["o"], rays["d"], tmax[:, None]], 1).astype(np.float32).tobytes())
        f.write(np.int32(len(light_tris)).tobytes())
        f.write(np.asarray(light_tris, np.int32).tobytes())
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(path), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    b = out.read_bytes()
    n, npx = rays.shape[0], W * H * 3
    o = 0
    rgb = np.frombuffer(b, np.uint8, npx, o).reshape(H, W, 3); o += npx
    rgb2 = np.frombuffer(b, np.uint8, npx, o).reshape(H, W, 3); o += npx
    ids = np.frombuffer(b, np.int32, n, o); o += 4 * n
    t = np.frombuffer(b, np.float32, n, o); o += 4 * n
    occ = np.frombuffer(b, np.uint8, n, o); o += n
    ids_b = np.frombuffer(b, np.int32, n, o); o += 4 * n
    t_b = np.frombuffer(b, np.float32, n, o); o += 4 * n
    occ_b = np.frombuffer(b, np.uint8, n, o)
    return rgb, rgb2, ids, t, occ, ids_b, t_b, occ_b


def scene_rays(rtlib, scene, n, seed):
    rng = np.random.default_rng(seed)
    v = scene["verts"].astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    o = rng.uniform(lo - 0.5 * (hi - lo), hi + 0.5 * (hi - lo), size=(n, 3))
    target = rng.uniform(lo, hi, size=(n, 3))
    d = target - o
    d /= np.linalg.norm(d, axis=1)[:, None]
    tmax = rng.uniform(0.1, 2.0, n) * np.linalg.norm(hi - lo)
    return rtlib.rays_array(o.astype(np.float32), d.astype(np.float32)), tmax.astype(np.float32)


CASES = ["ico-vertex-colour", "ico-aa2x2", "terrain-table-dir-spot", "ico-mirror-table", "ico-normals"]


def build_case(name):
    from raptor_gb300 import scenes
    if name.startswith("ico"):
        scene, frame = scenes.icosphere_scene(freq=8, res=96)
    else:
        scene, frame = scenes.terrain_scene(size_pow2=64, xres=120, yres=68)
    nt = scene["tris"].shape[0]
    mat = dict(frame["material"])
    aa = (1, 1)
    kinds = [0]
    mat_of_tri = np.zeros(nt, np.int32)
    materials = [mat]
    if name == "ico-aa2x2":
        aa = (2, 2)
    elif name == "terrain-table-dir-spot":
        # a phong_shader and an untextured coloured_mapper_shader, alternating
        m0 = dict(mat, flags=NO_VERTEX_COLOUR)
        m1 = dict(ka=(10.0, 5.0, 0.0), kd=(120.0, 200.0, 90.0), ks=(40.0, 40.0, 40.0), ns=8.0,
                  flags=NO_VERTEX_COLOUR)
        materials, kinds = [m0, m1], [1, 0]
        mat_of_tri = (np.arange(nt) % 3 == 0).astype(np.int32)
        c = frame["camera"]["pos"]
        frame = dict(frame, lights=[scenes.directional_light((-0.4, -0.8, -0.3)),
                                    scenes.spot_light((c[0] + 20.0, c[1] + 10.0, c[2] + 20.0), (0.7, -0.5, 0.5), 0.3,
                                                      0.6, rgb=(200.0, 180.0, 160.0))])
    elif name == "ico-mirror-table":
        m1 = dict(mat, rf=0.5)
        materials, kinds = [mat, m1], [0, 0]
        mat_of_tri = (scene["verts"][scene["tris"]][:, :, 1].max(1) > -0.999).astype(np.int32)   # the sphere mirrors
    elif name == "ico-normals":
        v = scene["verts"].astype(np.float64)
        n = v / np.maximum(np.linalg.norm(v, axis=1), 1e-9)[:, None]
        cn = n[scene["tris"]].astype(np.float32)
        ground = v[scene["tris"]][:, :, 1].max(1) < -0.999
        cn[ground] = np.float32(3.4028234663852886e38)
        scene = dict(scene, corner_normals=cn.reshape(nt, 9))
    return scene, frame, materials, kinds, mat_of_tri, aa


@pytest.mark.parametrize("name", CASES)
def test_adapter_frames_equal_c_abi(rtlib, ctx, oracle, adapter_exe, tmp_path, name):
    scene, frame, materials, kinds, mat_of_tri, aa = build_case(name)
    rays, tmax = scene_rays(rtlib, scene, 3000, seed=len(name))
    rgb, rgb2, ids, t, occ, ids_b, t_b, occ_b = run_adapter(adapter_exe, tmp_path, scene, frame, materials,
                                                            mat_of_tri, aa, rays, tmax, kinds)
    # the same frame through the C ABI
    sd = dict(scene)
    if len(materials) > 1:
        sd["mat_of_tri"] = mat_of_tri
    sc = rtlib.Scene(ctx, sd)
    if aa != (1, 1):
        want = sc.render_aa(frame, *aa)["rgb"]
    elif len(materials) > 1:
        want = sc.render(dict(frame, materials=materials))["rgb"]
    else:
        want = sc.render(dict(frame, material=materials[0]))["rgb"]
    assert np.array_equal(rgb, want)
    assert np.array_equal(rgb2, want)     # another ssd given: the adapter built its own gpu_bvh
    assert 0.05 < (rgb != np.asarray(frame["camera"]["background"], np.uint8)).any(-1).mean()
    # the ssd interface, one ray per call and batched, against the C ABI
    hits = sc.closest(rays)
    assert np.array_equal(ids, hits["tri"]) and np.array_equal(ids_b, hits["tri"])
    assert np.array_equal(t.view(np.uint32), hits["t"].view(np.uint32))
    assert np.array_equal(t_b.view(np.uint32), hits["t"].view(np.uint32))
    want_occ = sc.any(rtlib.rays_array(rays["o"], rays["d"], tmax))
    assert np.array_equal(occ, want_occ) and np.array_equal(occ_b, want_occ)
    assert 0.1 < (ids >= 0).mean() and 0 < want_occ.mean() < 1
    sc.close()
    # and the oracle, for the single-material pinhole frames
    if aa == (1, 1) and len(materials) == 1:
        ref = oracle.OracleScene(sd).render(dict(frame, material=materials[0]))
        within1, exact, maxd = pixel_agreement(rgb, ref["rgb"])
        assert within1 >= PIX_FRAC, (within1, exact, maxd)


@pytest.mark.parametrize("mirror", [False, True])
def test_render_image_is_the_reference_float_frame(rtlib, ctx, oracle, mirror):
    """rt_render_image returns the camera's float image (the colours
    ray_tracer stores with set_pixel): equal to the oracle's unclipped frame
    bit for bit on every pixel with the same primary hit, on host and device
    buffers alike, and clipped it is rt_render's RGB8 frame."""
    torch = pytest.importorskip("torch")
    from raptor_gb300 import scenes
    scene, frame = scenes.icosphere_scene(freq=8, res=96)
    if mirror:
        frame = dict(frame, materials=[dict(frame["material"], rf=0.5)])
    sc = rtlib.Scene(ctx, scene)
    out = sc.render_image(frame)
    st = out["stats"]
    assert st.status == 0 and st.primary_rays == 96 * 96
    img = out["fimg"]
    dev = torch.empty((96, 96, 3), dtype=torch.float32, device="cuda")
    sc.render_image(frame, fimg=dev)
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), img.view(np.uint32))
    rgb = sc.render(frame, want_ids=True)
    assert np.array_equal(np.clip(img, 0, 255).astype(np.uint8), rgb["rgb"])
    osc = oracle.OracleScene(scene)
    ref = osc.render(frame, want_ids=True, want_float=True)
    same = rgb["ids"] == ref["ids"]
    exact = (img.view(np.uint32) == ref["fimg"].view(np.uint32)).all(-1)
    assert exact[same].mean() >= 0.999, exact[same].mean()
    sc.close()


def soft_case(name):
    """The icosphere with a spherical light (radius 0.8), a quad light of two
    scene triangles and the sun; "mirror": the sphere reflects (rf 0.5);
    "diffuse": and spreads its reflection (rfd 0.2)."""
    from raptor_gb300 import scenes
    scene, frame = scenes.icosphere_scene(freq=8, res=80)
    scene, quad = scenes.add_area_light(scene, [(-0.9, 2.6, -0.9), (0.9, 2.6, -0.9), (0.9, 2.6, 0.9), (-0.9, 2.6, 0.9)],
                                        rgb=(255.0, 230.0, 200.0))
    nt = scene["tris"].shape[0]
    lights = [dict(frame["lights"][0], r=0.8), quad, scenes.directional_light((-0.4, -0.8, -0.3), rgb=(60.0, 60.0, 70.0))]
    mat = dict(frame["material"])
    materials, mat_of_tri = [mat], np.zeros(nt, np.int32)
    if name in ("mirror", "diffuse"):
        m1 = dict(mat, rf=0.5, rfd=0.2 if name == "diffuse" else 0.0)
        materials = [mat, m1]
        mat_of_tri = (scene["verts"][scene["tris"]][:, :, 1].max(1) > -0.999).astype(np.int32)
        mat_of_tri[-2:] = 0        # the light's triangles
    return scene, dict(frame, lights=lights), materials, mat_of_tri


@pytest.mark.parametrize("name", ["plain", "mirror"])
def test_adapter_soft_shadow_build(rtlib, ctx, tmp_path_factory, tmp_path, name):
    """The adapter compiled as part of a SOFT_SHADOW = 16 build: its frames
    are rt_render_distributed's with soft = 16 on the reference's stream --
    the first from position 0 (a fresh program), the second (another ssd)
    from where the first left it -- bit for bit; spherical, triangle-defined
    and directional lights, with and without mirror ray trees."""
    exe = compile_adapter(tmp_path_factory, ["SOFT_SHADOW=16"])
    scene, frame, materials, mat_of_tri = soft_case(name)
    rays, tmax = scene_rays(rtlib, scene, 100, seed=5)
    rgb, rgb2, *_ = run_adapter(exe, tmp_path, scene, frame, materials, mat_of_tri, (1, 1), rays, tmax,
                                [0] * len(materials))
    sd = dict(scene, mat_of_tri=mat_of_tri) if len(materials) > 1 else scene
    sc = rtlib.Scene(ctx, sd)
    f = dict(frame, materials=materials)
    a = sc.render_distributed(f, soft=16, offset=0)
    b = sc.render_distributed(f, soft=16, offset=a["stream_end"])
    assert np.array_equal(rgb, a["rgb"])
    assert np.array_equal(rgb2, b["rgb"])
    assert not np.array_equal(rgb, rgb2)      # the second frame drew new numbers
    sc.close()


def test_adapter_diffuse_build(rtlib, ctx, tmp_path_factory, tmp_path):
    """The adapter compiled as part of a SOFT_SHADOW = 16,
    DIFFUSE_REFLECTIONS = 16 build, with a diffuse mirror: per-pixel streams
    keyed 0 for the first frame and 1 for the second, as
    rt_render_distributed renders them."""
    exe = compile_adapter(tmp_path_factory, ["SOFT_SHADOW=16", "DIFFUSE_REFLECTIONS=16"])
    scene, frame, materials, mat_of_tri = soft_case("diffuse")
    rays, tmax = scene_rays(rtlib, scene, 100, seed=6)
    rgb, rgb2, *_ = run_adapter(exe, tmp_path, scene, frame, materials, mat_of_tri, (1, 1), rays, tmax, [0, 0])
    sc = rtlib.Scene(ctx, dict(scene, mat_of_tri=mat_of_tri))
    f = dict(frame, materials=materials)
    for got, seed in ((rgb, 0), (rgb2, 1)):
        want = sc.render_distributed(f, soft=16, diffuse=16, stream=rtlib.RT_STREAM_PIXEL, seed=seed)["rgb"]
        assert np.array_equal(got, want), seed
    sc.close()
