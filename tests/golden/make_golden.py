"""Regenerate the golden fixtures in this folder from the reference itself.

Run where the reference tree is present (x86-64 host):

    python tests/golden/make_golden.py [--ref /root/reference/RAPTor]

It writes
  bih_kats.json     traversal known-answer tests parsed from the reference's
                    raytracer/unit_tests/bih_tests.cc (6-triangle fixtures,
                    expected hit ids, distances and occlusion answers)
  morton_kats.json  Morton-code known answers parsed from
                    raytracer/unit_tests/vint_tests.cc
  ref_small.npz     inputs and outputs of the reference's own bvh,
                    ray_tracer() and clip_image_to_rgb() (compiled by
                    oracle/refbuild/Makefile) on small seeded scenes, also
                    with the camera's anti-aliasing factors (2x2, 3x2) and
                    with a reflective material
  ref_soft.npz      the reference built with soft shadows (SOFT_SHADOW =
                    16): the head of its random stream, its cosine table on
                    angles that reach every entry, and its soft-shadow frames
                    rendered one after another from a freshly started
                    generator (written by a fresh process, `--soft`)
The tests compare the C restatement (oracle/rtoracle.c) and the CUDA core
against these files; nothing at test time reads the reference tree.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

NUM = r"(-?[0-9.]+)f?"


def parse_bih_tests(path):
    src = open(path).read()
    tris = {"x": [], "y": [], "z": []}
    pt = r"point_t\(\s*" + NUM + r"\s*,\s*" + NUM + r"\s*,\s*" + NUM + r"\s*\)"
    for m in re.finditer(r"([xyz])_tris\.emplace_back\(mat\.get\(\),\s*" + pt + r",\s*" + pt + r",\s*" + pt, src):
        v = [float(m.group(i)) for i in range(2, 11)]
        tris[m.group(1)].append([v[0:3], v[3:6], v[6:9]])
    cases = []
    for m in re.finditer(r"BOOST_AUTO_TEST_CASE\(\s*(\w+)\s*\)\s*\{(.*?)\n\}", src, re.S):
        name, body = m.group(1), m.group(2)
        fx = re.search(r"bih uut\(([xyz])_tris", body)
        rr = re.search(r"ray r\(" + pt + r",\s*" + NUM + r",\s*" + NUM + r",\s*" + NUM + r"\)", body)
        if not fx or not rr:
            continue
        case = {"name": name, "fixture": fx.group(1),
                "origin": [float(rr.group(i)) for i in (1, 2, 3)],
                "dir": [float(rr.group(i)) for i in (4, 5, 6)]}
        fn = re.search(r"find_nearest_object\(&r, &h\)\s*==\s*(-?\d+)", body)
        if fn:
            case["nearest"] = int(fn.group(1))
        dc = re.search(r"BOOST_CHECK_CLOSE\(h\.d,\s*" + NUM, body)
        if dc:
            case["distance"] = float(dc.group(1))
        fo = re.search(r"BOOST_CHECK\((!?)uut\.found_nearer_object\(&r,\s*" + NUM + r"\)\)", body)
        if fo:
            case["nearer_t"] = float(fo.group(2))
            case["nearer"] = fo.group(1) != "!"
        cases.append(case)
    return {"source": "raytracer/unit_tests/bih_tests.cc", "tolerance_percent": 0.00001, "tris": tris,
            "cases": cases}


def parse_morton_tests(path):
    src = open(path).read()
    out = []
    vec = r"vfp_t\s+(\w+)\(([^;]*)\);"
    for m in re.finditer(r"BOOST_AUTO_TEST_CASE\(\s*(\w*morton_code_test)\s*\)\s*\{(.*?)\n\}", src, re.S):
        name, body = m.group(1), m.group(2)
        vals = {}
        for v in re.finditer(vec, body):
            parts = [p.strip() for p in v.group(2).split(",")]
            nums = []
            for p in parts:   # float literals, or "1.0f / 4.5f" evaluated in binary32 as C++ does
                terms = [np.float32(q.strip().rstrip("f")) for q in p.split("/")]
                val = terms[0] if len(terms) == 1 else np.float32(terms[0] / terms[1])
                nums.append(float(val))
            if len(nums) == 1:
                nums = nums * 4
            vals[v.group(1)] = nums
        exp = [int(e.group(2), 16) for e in re.finditer(r"mc\[(\d)\]\s*==\s*(0x[0-9a-fA-F]+)", body)]
        for i in range(4):
            out.append({"name": f"{name}[{i}]", "x": vals["x"][i], "y": vals["y"][i], "z": vals["z"][i],
                        "x_mul": vals["x_mul"][i], "y_mul": vals["y_mul"][i], "z_mul": vals["z_mul"][i],
                        "expected": exp[i]})
    return {"source": "raytracer/unit_tests/vint_tests.cc", "cases": out}


AA_FACTORS = ((2, 2), (3, 2))
REFLECTIVITY = {"ico": 0.5, "terrain": 0.35}
# glass-sphere frames (scenes.glass_scene keyword arguments): refraction with
# and without reflections, an index of 1, total internal reflection (2.4)
GLASS = ({}, {"ri": 1.0}, {"ri": 1.33, "tran": 0.9, "rf_glass": 0.0},
         {"ri": 2.4, "tran": 0.5, "rf_glass": 0.5, "rf_ground": 0.0})
# tone-mapped frames: (camera::tone_map arguments + gamma, anti-aliasing factors)
TONE = (({"mode": 0}, (1, 1)), ({"mode": 1}, (1, 1)), ({"mode": 4, "gamma": 2.2}, (1, 1)),
        ({"mode": 5}, (1, 1)), ({"mode": 6}, (1, 1)), ({"mode": 7, "gamma": 1.8}, (1, 1)),
        ({"mode": 9}, (1, 1)), ({"mode": 4, "desaturate": True, "key": 0.5}, (1, 1)),
        ({"mode": 5, "stretch": True}, (1, 1)), ({"mode": 1, "desaturate": True, "stretch": True, "gamma": 2.2}, (2, 2)),
        ({"mode": 9, "desaturate": True, "stretch": True, "gamma": 1.0}, (3, 2)), ({"mode": 0, "gamma": 2.2}, (1, 1)),
        ({"mode": 7, "key": 0.3, "stretch": True}, (2, 1)))


def small_scenes():
    from raptor_gb300 import scenes
    out = {}
    s, f = scenes.icosphere_scene(freq=8, seed=0, res=64)
    out["ico"] = (s, f)
    h = scenes.diamond_square(32, 0.55, 1)
    v, t, hs = scenes.heightfield_mesh(h, 64.0, 12.0)
    col = scenes.slope_colours(hs, 2.0, 12.0)
    s2 = scenes._pack(v, t, col)
    f2 = {"camera": scenes.look_at_camera((0.0, 30.0, 0.0), (32.0, 6.0, 32.0), 60.0, 64, 48, (110.0, 160.0, 230.0)),
          "lights": [scenes.directional_light((-0.4, -0.8, -0.3))], "material": dict(scenes.DEFAULT_MATERIAL)}
    out["terrain"] = (s2, f2)
    return out


def soup(seed=7, n=300):
    """Random triangle soup with some light/transparent triangles."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-5, 5, (n, 3))
    v = (c[:, None, :] + rng.uniform(-1, 1, (n, 3, 3))).reshape(-1, 3)
    t = np.arange(3 * n, dtype=np.int32).reshape(-1, 3)
    flags = np.zeros(n, np.uint32)
    flags[rng.uniform(size=n) < 0.1] = 1
    flags[rng.uniform(size=n) < 0.1] |= 2
    o = rng.uniform(-8, 8, (4000, 3))
    d = rng.normal(size=(4000, 3))
    d = d / np.sqrt((d ** 2).sum(1))[:, None]
    tmax = rng.uniform(0.5, 12.0, 4000)
    return ({"verts": v.astype(np.float32), "tris": t, "vattr": None, "flags": flags},
            o.astype(np.float32), d.astype(np.float32), tmax.astype(np.float32))


# tone maps applied by the reference to fixed float frames (the histogram
# modes need a wide luminance range: a dark ambient term, a strong specular
# highlight and a dim coloured light on the icosphere)
FRAME_TONE = (({"mode": 2}, (1, 1)), ({"mode": 3}, (1, 1)),
              ({"mode": 3, "desaturate": True, "stretch": True, "gamma": 2.2}, (2, 2)),
              ({"mode": 2, "stretch": True, "gamma": 1.8}, (3, 2)), ({"mode": 3, "gamma": 2.2}, (2, 1)),
              ({"mode": 5, "gamma": 2.2}, (1, 1)), ({"mode": 9, "desaturate": True}, (2, 2)))


def spot_frames():
    """The icosphere lit by spot lights (light.h:24-25, 49-55): narrow and
    wide cones, a coloured one with distance fall-off beside a point light."""
    from raptor_gb300 import scenes
    s, f = scenes.icosphere_scene(freq=8, seed=0, res=64)
    sets = ([scenes.spot_light((0.0, 4.0, 1.0), (0.0, 1.0, 0.25), 0.2, 0.6)],
            [scenes.spot_light((2.0, 3.0, 2.0), (0.5, 0.6, 0.5), 0.1, 0.3, rgb=(255.0, 200.0, 100.0), d=0.05),
             scenes.point_light((-3.0, 4.0, 2.0), rgb=(60.0, 60.0, 90.0))],
            [scenes.spot_light((0.0, 2.0, 3.0), (0.0, 0.5, 1.0), 0.0, 1.2)])
    return s, [dict(f, lights=ls) for ls in sets]


def hdr_frame():
    from raptor_gb300 import scenes
    s, f = scenes.icosphere_scene(freq=8, seed=0, res=64)
    f = dict(f, material=dict(f["material"], ka=(0.4, 0.4, 0.4), ks=(255.0, 255.0, 255.0), ns=30.0),
             lights=[scenes.point_light((3.0, 5.0, 3.0)),
                     scenes.point_light((-2.0, 0.5, 1.5), rgb=(40.0, 30.0, 255.0), d=0.3)])
    return s, f


def _polygons(rng):
    """Faces for the parser cases: convex and concave polygons, collinear
    vertices, a star, as (vertex list, face list) in the plane z = const."""
    verts, faces = [], []

    def add(pts):
        base = len(verts)
        verts.extend(pts)
        faces.append(list(range(base, base + len(pts))))

    for k, n in enumerate((4, 5, 6, 7, 9)):
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        r = rng.uniform(0.5, 1.5, n)
        add([(float(np.cos(a) * q + 3 * k), float(np.sin(a) * q), 0.25 * k) for a, q in zip(ang, r)])
    add([(0, 0, 2), (2, 0, 2), (2, 1, 2), (1, 1, 2), (1, 2, 2), (0, 2, 2)])                # L shape
    add([(0, 0, 3), (1, 0, 3), (2, 0, 3), (2, 1, 3), (0, 1, 3)])                           # collinear vertex
    star = []
    for i in range(10):
        rr = 1.0 if i % 2 == 0 else 0.4
        star.append((float(rr * np.cos(np.pi * i / 5) + 6), float(rr * np.sin(np.pi * i / 5)), 4.0))
    add(star)
    add([(0, 0, 5), (0.5, 0.2, 5), (1, 0, 5), (1, 1, 5), (0.5, 0.8, 5), (0, 1, 5)])       # two notches
    return verts, faces


def mesh_frame(tris):
    """A camera looking at the bounding box of the parsed triangles from
    above and in front, with one point light and one directional light."""
    from raptor_gb300 import scenes
    v = tris.reshape(-1, 3).astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    c = (lo + hi) / 2
    size = float(np.max(hi - lo))
    eye = c + np.array([0.1 * size, 0.6 * size, 1.2 * size])
    cam = scenes.look_at_camera(tuple(eye), tuple(c), 50.0, 96, 64, background=(30.0, 40.0, 60.0))
    lights = [scenes.point_light(tuple(c + np.array([0.3 * size, 1.0 * size, 0.8 * size]))),
              scenes.directional_light((-0.3, -0.9, -0.2), rgb=(90.0, 90.0, 90.0))]
    return {"camera": cam, "lights": lights}


def mesh_files():
    """(name, kind 1 OFF / 2 PLY, file bytes) for the parser cases."""
    import struct
    from raptor_gb300 import scenes
    rng = np.random.default_rng(11)
    sv, st = scenes.geodesic_sphere(3)
    pv, pf = _polygons(rng)
    verts = [tuple(float(x) for x in v) for v in sv] + [(x * 0.5 + 5.0, y * 0.5, z * 0.5) for x, y, z in pv]
    faces = [list(map(int, t)) for t in st] + [[i + len(sv) for i in f] for f in pf]
    out = []
    # OFF, LF and CRLF line ends, padded fields
    for name, nl in (("off_lf", "\n"), ("off_crlf", "\r\n")):
        lines = ["OFF", f"{len(verts)} {len(faces)} 0"]
        lines += [f"{x!r} {y!r}  {z!r}" if i % 3 else f"  {x:.9g}\t{y:.9g} {z:.9g}" for i, (x, y, z) in enumerate(verts)]
        lines += [" ".join([str(len(f))] + [str(i) for i in f]) for f in faces]
        out.append((name, 1, (nl.join(lines) + nl).encode()))
    # PLY ascii: comments, normals and colours on the vertices, degenerate triangles
    dverts = verts + [(9.0, 9.0, 9.0), (9.0, 9.0, 9.0), (10.0, 9.0, 9.0), (11.0, 9.0, 9.0)]
    dfaces = faces + [[len(verts), len(verts) + 1, len(verts) + 2], [len(verts), len(verts) + 2, len(verts) + 3]]
    hdr = ["ply", "format ascii 1.0", "comment made by the parser tests", f"element vertex {len(dverts)}",
           "property float x", "property float y", "property float z", "property float nx", "property float ny",
           "property float nz", "property uchar red", "property uchar green", "property uchar blue",
           f"element face {len(dfaces)}", "property list uchar int vertex_indices", "end_header"]
    body = [f"{x!r} {y!r} {z!r} 0 0 1 {i % 256} 7 9" for i, (x, y, z) in enumerate(dverts)]
    body += [" ".join([str(len(f))] + [str(i) for i in f]) for f in dfaces]
    out.append(("ply_ascii", 2, ("\n".join(hdr + body) + "\n").encode()))
    # PLY binary big endian: vertex colour + normal + an extra float, face
    # intensity before and colour + an extra uchar after the index list
    hdr = ["ply", "format binary_big_endian 1.0", "obj_info synthetic", f"element vertex {len(dverts)}",
           "property float x", "property float y", "property float z", "property uchar red",
           "property uchar green", "property uchar blue", "property float nx", "property float ny",
           "property float nz", "property float confidence", f"element face {len(dfaces)}",
           "property uchar intensity", "property list uchar int vertex_indices", "property uchar red",
           "property uchar green", "property uchar blue", "property uchar flags", "end_header"]
    data = bytearray(("\n".join(hdr) + "\n").encode())
    for i, (x, y, z) in enumerate(dverts):
        data += struct.pack(">fff", x, y, z) + bytes([i % 256, 3, 5]) + struct.pack(">ffff", 0, 0, 1, 0.5)
    palette = [(200, 10, 10), (10, 200, 10), (10, 10, 200), (90, 90, 90)]
    for k, f in enumerate(dfaces):
        data += bytes([17]) + bytes([len(f)]) + struct.pack(f">{len(f)}i", *f) + bytes(palette[k % 4]) + bytes([1])
    out.append(("ply_binary", 2, bytes(data)))
    # OBJ: v / vt / vn, faces as v, v/t, v//n and v/t/n with negative
    # (relative) indices, usemtl groups, g / o / s lines, comments, CRLF
    for name, nl in (("obj_lf", "\n"), ("obj_crlf", "\r\n")):
        lines = ["# synthetic OBJ for the parser tests", "o scene", "g sphere"]
        lines += [f"v {x!r} {y!r} {z!r}" for x, y, z in dverts]
        lines += [f"vt {float(i % 7) / 7!r} {float(i % 5) / 5!r}" for i in range(len(dverts))]
        lines += [f"vn {x!r} {y!r} {z + 0.5!r}" for x, y, z in dverts]
        mats = ["stone", "glass", "stone", "metal"]
        for k, f in enumerate(dfaces):
            if k % 37 == 0:
                lines.append(f"usemtl {mats[(k // 37) % 4]}")
            if k % 50 == 0:
                lines.append(f"s {k % 2}")
            form = k % 4
            if form == 0:
                toks = [str(i + 1) for i in f]
            elif form == 1:
                toks = [f"{i + 1}/{i + 1}" for i in f]
            elif form == 2:
                toks = [f"{i - len(dverts)}//{i + 1}" for i in f]
            else:
                toks = [f"{i + 1}/{i - len(dverts)}/{i - len(dverts)}" for i in f]
            lines.append("f " + " ".join(toks))
        out.append((name, 3, (nl.join(lines) + nl).encode()))
    return out


def soft_cases():
    """(name, scene, frame) of the soft-shadow fixtures: spherical point
    lights of several radii, one with a directional light beside it, a spot
    light with a radius, a terrain, and triangle-defined lights: a quad (two
    triangles, so 17 rays made for 16), a spot-light disk of 12 triangles
    beside a spherical light, and a 9-triangle disk over the terrain (the
    binary32 stride decides which triangles get a second ray)."""
    from raptor_gb300 import scenes
    s, f = scenes.icosphere_scene(freq=8, res=96)
    pl = dict(f["lights"][0], r=0.8)
    sun = scenes.directional_light((-0.4, -0.8, -0.3))
    spot = dict(scenes.spot_light((2.0, 4.0, 2.0), (-0.4, -0.8, -0.4), 0.2, 0.5), r=0.6)
    t, tf = scenes.terrain_scene(size_pow2=64, xres=120, yres=68)
    sq, quad = scenes.add_area_light(s, [(-0.9, 2.6, -0.9), (0.9, 2.6, -0.9), (0.9, 2.6, 0.9), (-0.9, 2.6, 0.9)],
                                     rgb=(255.0, 230.0, 200.0))
    sd, disk = scenes.add_area_light(s, scenes.regular_polygon((1.5, 3.0, 1.5), 0.8, 14, 0.4),
                                     spot=((-0.45, -0.8, -0.4), 0.25, 0.6))
    td, tdisk = scenes.add_area_light(t, scenes.regular_polygon((520.0, 330.0, 480.0), 60.0, 11, 0.3),
                                      rgb=(255.0, 240.0, 220.0))
    return [("ico-point", s, dict(f, lights=[pl])),
            ("ico-point-dir", s, dict(f, lights=[pl, sun])),
            ("ico-spot-point", s, dict(f, lights=[spot, dict(pl, pos=(-3.0, 4.0, 1.0), r=1.5)])),
            ("terrain-point-dir", t, dict(tf, lights=[dict(scenes.point_light((300.0, 260.0, 500.0)), r=40.0),
                                                      tf["lights"][0]])),
            ("ico-quad-light", sq, dict(f, lights=[quad])),
            ("ico-disk-spot-point", sd, dict(f, lights=[disk, dict(pl, pos=(-3.0, 4.0, 1.0), r=1.0)])),
            ("terrain-disk-dir", td, dict(tf, lights=[tdisk, tf["lights"][0]]))]


def soft_main():
    """ref_soft.npz, in a process whose reference generator is untouched."""
    import ctypes as C
    import oracle as O
    lib = O.ref_soft_lib()
    samples = lib["rref_soft_shadow_samples"]()
    arrays = {"samples": np.array([samples], np.int32)}
    head = np.empty(4096, np.float32)
    lib["rref_random"](head.shape[0], head.ctypes.data_as(C.POINTER(C.c_float)))
    arrays["stream_head"] = head
    n = 16384
    ang = np.concatenate([(np.arange(n, dtype=np.float64) + 0.5) * (2 * np.pi / n),
                          np.random.default_rng(5).uniform(-20.0, 20.0, 20000)]).astype(np.float32)
    arrays["lut_angles"] = ang
    arrays["lut_cos"] = np.array([lib["rref_lut_cos"](float(a)) for a in ang], np.float32)
    arrays["lut_sin"] = np.array([lib["rref_lut_sin"](float(a)) for a in ang], np.float32)
    offset = head.shape[0]
    cases = soft_cases()
    for k, (name, s, f) in enumerate(cases):
        arrays[f"soft{k}_rgb"] = O.RefScene(s, f["material"], soft=True).render(f)["rgb"]
        arrays[f"soft{k}_frame"] = np.frombuffer(json.dumps(f).encode(), np.uint8)
        arrays[f"soft{k}_scene"] = np.frombuffer(json.dumps(name).encode(), np.uint8)
        arrays[f"soft{k}_offset"] = np.array([offset], np.int64)
        for key in ("verts", "tris", "vattr", "flags"):
            if s.get(key) is not None:
                arrays[f"soft{k}_{key}"] = s[key]
        # the stream position after the frame, as the restatement counts it
        offset = O.OracleScene(s).render_soft(f, samples, offset, threads=os.cpu_count() or 1)["stream_end"]
        print(f"soft frame {name}: stream {int(arrays[f'soft{k}_offset'][0])} -> {offset}")
    # the reference's generator stands exactly where the restatement says
    tail = np.empty(64, np.float32)
    lib["rref_random"](64, tail.ctypes.data_as(C.POINTER(C.c_float)))
    if not np.array_equal(tail, O.ref_random(offset, 64)):
        raise SystemExit("soft-shadow stream accounting differs from the reference")
    arrays["stream_end"] = np.array([offset], np.int64)
    np.savez_compressed(os.path.join(HERE, "ref_soft.npz"), **arrays)
    print("wrote ref_soft.npz")


def dist_cases():
    """(name, scene, frame, diffuse) of the distributed-ray-tracing
    fixtures: ray trees (mirror and glass) with soft shadows from the
    SOFT_SHADOW = 16 build (diffuse False), and diffuse reflections and
    refractions from the SOFT_SHADOW = 16, DIFFUSE_REFLECTIONS = 16 build
    (diffuse True)."""
    from raptor_gb300 import scenes
    g, gf = scenes.glass_scene(freq=8, res=64)
    glights = [dict(gf["lights"][0], r=0.7), gf["lights"][1]]
    gq, quad = scenes.add_area_light(g, [(1.5, 3.0, 1.5), (3.0, 3.0, 1.5), (3.0, 3.4, 3.0), (1.5, 3.4, 3.0)])
    ico, fi = scenes.icosphere_scene(freq=8, res=72)
    # off the sphere's symmetry plane x = 0, where mirror rays would run
    # along edges (ties in secondary hits)
    fi = dict(fi, camera=scenes.look_at_camera((0.013, 0.5, 4.0), (0.0, 0.0, 0.0), 60.0, 72, 72))
    mirror = [dict(fi["material"], rf=0.5)]
    ico = dict(ico, mat_of_tri=np.zeros(ico["tris"].shape[0], np.int32))
    dm = [dict(gf["materials"][0], rfd=0.2), dict(gf["materials"][1], rfd=0.1, td=0.05)]
    ishiny = [dict(fi["material"], rf=0.6, rfd=0.3)]
    spot = dict(scenes.spot_light((2.0, 4.0, 2.0), (-0.4, -0.8, -0.4), 0.2, 0.5), r=0.6)
    iq, iquad = scenes.add_area_light(ico, [(-0.9, 2.6, -0.9), (0.9, 2.6, -0.9), (0.9, 2.6, 0.9), (-0.9, 2.6, 0.9)])
    return [("glass-soft", g, dict(gf, lights=glights), False),
            ("glass-quad-light", gq, dict(gf, lights=[quad, gf["lights"][1]]), False),
            ("ico-mirror-spot", ico, dict(fi, lights=[spot, dict(fi["lights"][0], r=0.8)], materials=mirror,
                                          material=mirror[0]), False),
            ("glass-diffuse", g, dict(gf, lights=glights, materials=dm, material=dm[0]), True),
            ("ico-diffuse-quad", iq, dict(fi, lights=[iquad, spot], materials=ishiny, material=ishiny[0]), True)]


def dist_main():
    """ref_distributed.npz, in a process whose reference generators are
    untouched: each build's frames rendered one after another."""
    import ctypes as C
    import oracle as O
    arrays = {"soft": np.array([O.REF_SOFT_SAMPLES], np.int32), "diffuse": np.array([O.REF_DIFFUSE_SAMPLES], np.int32)}
    offset = {False: 0, True: 0}
    for k, (name, s, f, diffuse) in enumerate(dist_cases()):
        arrays[f"dist{k}_rgb"] = O.RefScene(s, f["materials"], soft=not diffuse, diffuse=diffuse).render(f)["rgb"]
        arrays[f"dist{k}_frame"] = np.frombuffer(json.dumps(f).encode(), np.uint8)
        arrays[f"dist{k}_name"] = np.frombuffer(json.dumps(name).encode(), np.uint8)
        arrays[f"dist{k}_diffuse"] = np.array([O.REF_DIFFUSE_SAMPLES if diffuse else 0], np.int32)
        arrays[f"dist{k}_offset"] = np.array([offset[diffuse]], np.int64)
        for key in ("verts", "tris", "vattr", "flags", "mat_of_tri"):
            if s.get(key) is not None:
                arrays[f"dist{k}_{key}"] = s[key]
        out = O.OracleScene(s).render_distributed(f, soft=O.REF_SOFT_SAMPLES,
                                                  diffuse=O.REF_DIFFUSE_SAMPLES if diffuse else 0,
                                                  offset=offset[diffuse])
        print(f"distributed frame {name}: stream {offset[diffuse]} -> {offset[diffuse] + out['drawn']}")
        offset[diffuse] += out["drawn"]
    for diffuse, lib in ((False, O.ref_soft_lib()), (True, O.ref_diffuse_lib())):
        tail = np.empty(64, np.float32)
        lib["rref_random"](64, tail.ctypes.data_as(C.POINTER(C.c_float)))
        if not np.array_equal(tail, O.ref_random(offset[diffuse], 64)):
            raise SystemExit("distributed stream accounting differs from the reference")
    arrays["stream_end"] = np.array([offset[False], offset[True]], np.int64)
    np.savez_compressed(os.path.join(HERE, "ref_distributed.npz"), **arrays)
    print("wrote ref_distributed.npz")


def bilateral_cases():
    """(name, float frame, camera, tone, aa) of the bilateral tone-map
    fixtures: rendered float frames dimmed so the reference's bilateral
    mode, which does not subtract the base's maximum, keeps contrast; no
    pixel at or below the reference's 3.18e-7 luminance floor (the
    reference reads an unset value there)."""
    import oracle as O
    from raptor_gb300 import scenes
    out = []
    t, tf = scenes.terrain_scene(size_pow2=128, xres=320, yres=180)
    tf = dict(tf, camera=dict(tf["camera"], background=(40.0, 60.0, 90.0)))
    tfimg = O.OracleScene(t).render(tf, want_float=True)["fimg"]
    out.append(("terrain320", (tfimg * np.float32(0.01)).astype(np.float32), tf["camera"], {"mode": 8}, (1, 1)))
    out.append(("terrain320-gamma", (tfimg * np.float32(0.01)).astype(np.float32), tf["camera"],
                {"mode": 8, "gamma": 2.2}, (1, 1)))
    g, gf = scenes.glass_scene(freq=8, res=96)
    gfimg = O.OracleScene(g).render(gf, want_float=True)["fimg"]
    out.append(("glass96-gamma", (gfimg * np.float32(1.0 / 300.0)).astype(np.float32), gf["camera"],
                {"mode": 8, "gamma": 2.2}, (1, 1)))
    a, af = scenes.glass_scene(freq=8, res=64)
    ss = O.supersampled(af, 2, 2)
    afimg = O.OracleScene(a).render(ss, want_float=True)["fimg"]
    out.append(("glass64-aa2x2", (afimg * np.float32(1.0 / 300.0)).astype(np.float32), af["camera"],
                {"mode": 8, "gamma": 2.2, "stretch": True}, (2, 2)))
    return out


def bilateral_main():
    """ref_bilateral.npz: the reference's bilateral tone mapper
    (camera::bilateral_filter_tone_map) on fixed float frames, its FFTW
    calls served by the harness's transforms."""
    import oracle as O
    arrays = {}
    for k, (name, fimg, cam, tone, aa) in enumerate(bilateral_cases()):
        arrays[f"bil{k}_fimg"] = fimg
        arrays[f"bil{k}_rgb"] = O.ref_tone_map_image(fimg, cam, tone, aa)
        arrays[f"bil{k}_args"] = np.frombuffer(json.dumps({"name": name, "camera": cam, "tone": tone,
                                                           "aa": list(aa)}).encode(), np.uint8)
        print(f"bilateral {name}: std {arrays[f'bil{k}_rgb'].std():.1f}")
    np.savez_compressed(os.path.join(HERE, "ref_bilateral.npz"), **arrays)
    print("wrote ref_bilateral.npz")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("RAPTOR_REF", "/root/reference/RAPTor"))
    ap.add_argument("--soft", action="store_true", help="write only ref_soft.npz (needs a fresh process)")
    ap.add_argument("--dist", action="store_true", help="write only ref_distributed.npz (needs a fresh process)")
    ap.add_argument("--bilateral", action="store_true", help="write only ref_bilateral.npz")
    a = ap.parse_args()
    if a.bilateral:
        import oracle as O
        O.build()
        return bilateral_main()
    if a.soft:
        import oracle as O
        O.build()
        return soft_main()
    if a.dist:
        import oracle as O
        O.build()
        return dist_main()
    kats = parse_bih_tests(os.path.join(a.ref, "raytracer/unit_tests/bih_tests.cc"))
    json.dump(kats, open(os.path.join(HERE, "bih_kats.json"), "w"), indent=1)
    mort = parse_morton_tests(os.path.join(a.ref, "raytracer/unit_tests/vint_tests.cc"))
    json.dump(mort, open(os.path.join(HERE, "morton_kats.json"), "w"), indent=1)
    print(f"bih KATs: {len(kats['cases'])}, morton KATs: {len(mort['cases'])}")

    import oracle as O
    O.build()
    if not O.ref_available():
        raise SystemExit("reference harness not built (needs the reference tree on an x86-64 host)")
    arrays = {}
    for key, (s, f) in small_scenes().items():
        rs = O.RefScene(s, f["material"])
        og, dr = O.camera_rays(f["camera"], lib=O.ref_lib())
        ids, t, u, v = rs.closest(og, dr)
        rgb = rs.render(f)["rgb"]
        arrays.update({f"{key}_verts": s["verts"], f"{key}_tris": s["tris"], f"{key}_vattr": s["vattr"],
                       f"{key}_ray_o": og, f"{key}_ray_d": dr, f"{key}_id": ids, f"{key}_t": t, f"{key}_u": u,
                       f"{key}_v": v, f"{key}_rgb": rgb})
        # anti-aliased frames: the camera's x_a_res / y_a_res factors
        for ax, ay in AA_FACTORS:
            arrays[f"{key}_aa{ax}{ay}_rgb"] = rs.render(f, aa=(ax, ay))["rgb"]
        # a reflective material: mirror rays while their power exceeds 0.1
        mat = dict(f["material"], rf=REFLECTIVITY[key])
        fr = dict(f, material=mat)
        arrays[f"{key}_refl_rf"] = np.array([REFLECTIVITY[key]], np.float32)
        arrays[f"{key}_refl_rgb"] = O.RefScene(s, mat).render(fr)["rgb"]
        arrays[f"{key}_frame"] = np.frombuffer(json.dumps(f).encode(), dtype=np.uint8)
        # tone mapping and gamma (camera::tone_map, camera::gamma_correct)
        for k, (tone, aa) in enumerate(TONE):
            arrays[f"{key}_tone{k}_rgb"] = rs.render(f, aa=aa, tone=tone)["rgb"]
    # the reference's tone maps on fixed float frames (the restatement's
    # render of the HDR icosphere on each anti-aliasing grid)
    hs, hf = hdr_frame()
    osc = O.OracleScene(hs)
    for k, (tone, aa) in enumerate(FRAME_TONE):
        fimg = osc.render(O.supersampled(hf, *aa), want_float=True)["fimg"]
        arrays[f"ftone{k}_fimg"] = fimg.astype(np.float32)
        arrays[f"ftone{k}_rgb"] = O.ref_tone_map_image(fimg, hf["camera"], tone, aa)
    arrays["ftone_cases"] = np.frombuffer(json.dumps([[t, list(aa)] for t, aa in FRAME_TONE]).encode(), np.uint8)
    arrays["ftone_camera"] = np.frombuffer(json.dumps(hf["camera"]).encode(), np.uint8)
    # spot lights
    ss, sframes = spot_frames()
    rs = O.RefScene(ss, sframes[0]["material"])
    for k, fr in enumerate(sframes):
        arrays[f"spot{k}_rgb"] = rs.render(fr)["rgb"]
        arrays[f"spot{k}_frame"] = np.frombuffer(json.dumps(fr).encode(), np.uint8)
    # per-triangle materials with refraction: the glass sphere
    from raptor_gb300 import scenes
    for k, kw in enumerate(GLASS):
        s, f = scenes.glass_scene(**kw)
        arrays[f"glass{k}_rgb"] = O.RefScene(s, f["materials"]).render(f)["rgb"]
        arrays[f"glass{k}_args"] = np.frombuffer(json.dumps(kw).encode(), dtype=np.uint8)
        if k == 0:
            for j, (tone, aa) in enumerate(TONE):
                arrays[f"glass0_tone{j}_rgb"] = O.RefScene(s, f["materials"]).render(f, aa=aa, tone=tone)["rgb"]
    arrays["tone_cases"] = np.frombuffer(json.dumps([[t, list(aa)] for t, aa in TONE]).encode(), dtype=np.uint8)
    # scene ingest: the reference's own OFF and PLY parsers
    import tempfile
    cases = mesh_files()
    with tempfile.TemporaryDirectory() as td:
        for k, (name, kind, data) in enumerate(cases):
            path = os.path.join(td, f"{name}.{('off', 'ply', 'obj')[kind - 1]}")
            open(path, "wb").write(data)
            tris, nmat = O.ref_parse_mesh(path, kind)
            # the reference's own render of the parsed scene (its parser's
            # phong materials), for the ingest -> render parity test
            frame = mesh_frame(tris)
            arrays[f"mesh{k}_render_rgb"] = O.ref_parse_and_render(path, kind, frame)
            arrays[f"mesh{k}_frame"] = np.frombuffer(json.dumps(frame).encode(), np.uint8)
            arrays[f"mesh{k}_bytes"] = np.frombuffer(data, np.uint8)
            arrays[f"mesh{k}_kind"] = np.array([kind], np.int32)
            arrays[f"mesh{k}_tris"] = tris
            arrays[f"mesh{k}_nmat"] = np.array([nmat], np.int32)
            print(f"mesh {name}: {tris.shape[0]} triangles, {nmat} materials")
    s, o, d, tmax = soup()
    rs = O.RefScene(s, dict(__import__("raptor_gb300.scenes", fromlist=["x"]).DEFAULT_MATERIAL))
    ids, t, u, v = rs.closest(o, d)
    occ = rs.any(o, d, tmax)
    arrays.update({"soup_verts": s["verts"], "soup_tris": s["tris"], "soup_flags": s["flags"], "soup_ray_o": o,
                   "soup_ray_d": d, "soup_tmax": tmax, "soup_id": ids, "soup_t": t, "soup_u": u, "soup_v": v,
                   "soup_occ": occ})
    np.savez_compressed(os.path.join(HERE, "ref_small.npz"), **arrays)
    print("wrote ref_small.npz:", {k: v.shape for k, v in arrays.items()})
    # the soft-shadow fixtures need the reference's generator untouched
    import subprocess
    subprocess.run([sys.executable, os.path.abspath(__file__), "--soft", "--ref", a.ref], check=True)


if __name__ == "__main__":
    main()
