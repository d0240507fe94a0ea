"""Soft shadows (rt_render_soft_shadows) against the reference built with
SOFT_SHADOW = 16 (tests/golden/ref_soft.npz: frames rendered one after
another from a freshly started generator) and against the oracle's
restatement (oracle/rtoracle.c, ro_render_soft) on larger frames, up to the
headline terrain.

The random points are the reference's own stream, so frames are compared
pixel for pixel: every pixel equal except those whose camera ray passes
within 1e-5 of a triangle edge (ties, tests/parity.py), and the stream
position after each frame equal to the reference's."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from parity import PIX_FRAC, edge_distance, pixel_agreement

pytestmark = pytest.mark.gpu

NTHREADS = max(1, os.cpu_count() or 1)


@pytest.fixture(scope="module")
def soft_golden():
    return np.load(os.path.join(GOLDEN, "ref_soft.npz"))


def golden_cases(g):
    k = 0
    while f"soft{k}_rgb" in g.files:
        frame = json.loads(g[f"soft{k}_frame"].tobytes().decode())
        scene = {"verts": g[f"soft{k}_verts"], "tris": g[f"soft{k}_tris"], "vattr": g[f"soft{k}_vattr"]}
        if f"soft{k}_flags" in g.files:
            scene["flags"] = g[f"soft{k}_flags"]
        nxt = int(g[f"soft{k + 1}_offset"][0]) if f"soft{k + 1}_offset" in g.files else int(g["stream_end"][0])
        yield k, scene, frame, int(g[f"soft{k}_offset"][0]), nxt, g[f"soft{k}_rgb"]
        k += 1


def edge_pixels(oracle, scene, frame, ids):
    o, d = oracle.camera_rays(frame["camera"])
    H, W = frame["camera"]["yres"], frame["camera"]["xres"]
    return (edge_distance(scene["verts"], scene["tris"], ids.reshape(-1), o, d) < 1e-5).reshape(H, W)


def test_soft_shadows_match_reference(rtlib, ctx, oracle, soft_golden):
    """The reference's own soft-shadow frames, each from the stream position
    the reference had reached: equal on every pixel but edge ties, and the
    stream position after each frame the reference's."""
    samples = int(soft_golden["samples"][0])
    for k, scene, frame, offset, nxt, ref in golden_cases(soft_golden):
        sc = rtlib.Scene(ctx, scene)
        out = sc.render_soft(frame, samples, offset)
        assert out["stats"].status == 0
        assert out["stream_end"] == nxt, (k, out["stream_end"], nxt)
        ids = sc.render(dict(frame, lights=[]), want_ids=True)["ids"]
        diff = np.abs(out["rgb"].astype(int) - ref.astype(int)).max(-1) > 0
        near = edge_pixels(oracle, scene, frame, ids)
        assert not (diff & ~near).any(), (k, np.argwhere(diff & ~near)[:5])
        nsph = sum(1 for l in frame["lights"] if l["kind"] != 1)
        hits = int((ids >= 0).sum())
        assert out["stats"].secondary_rays == hits * (nsph * samples + (len(frame["lights"]) - nsph))
        sc.close()


def test_soft_shadows_match_oracle_float_frames(rtlib, ctx, oracle):
    """480x270 terrain with a spherical light (radius 40) beside the sun,
    8 samples, from a nonzero stream position: the float image equals the
    oracle's bit for bit on every pixel with the same primary hit."""
    from raptor_gb300 import scenes
    scene, frame = scenes.terrain_scene(size_pow2=256, xres=480, yres=270)
    frame = dict(frame, lights=[dict(scenes.point_light((300.0, 260.0, 500.0)), r=40.0), frame["lights"][0]])
    sc = rtlib.Scene(ctx, scene)
    out = sc.render_soft(frame, 8, 12345, want_float=True)
    ref = oracle.OracleScene(scene).render_soft(frame, 8, 12345, threads=NTHREADS, want_ids=True, want_float=True)
    assert out["stream_end"] == ref["stream_end"]
    ids = sc.render(dict(frame, lights=[]), want_ids=True)["ids"]
    same = ids == ref["ids"]
    exact = (out["fimg"].view(np.uint32) == ref["fimg"].view(np.uint32)).all(-1)
    assert exact[same].mean() == 1.0, exact[same].mean()
    assert np.array_equal(np.clip(out["fimg"], 0, 255).astype(np.uint8), out["rgb"])
    # partly lit pixels exist (the penumbra)
    hard = sc.render_image(frame)["fimg"]
    assert (np.abs(hard - out["fimg"]).max(-1) > 1.0).mean() > 0.01
    sc.close()


def test_soft_shadows_one_sample_is_the_hard_frame(rtlib, ctx):
    """samples = 1 draws no numbers and gives rt_render_image's frame."""
    from raptor_gb300 import scenes
    scene, frame = scenes.icosphere_scene(freq=16, res=128)
    frame = dict(frame, lights=[dict(frame["lights"][0], r=0.7)])
    sc = rtlib.Scene(ctx, scene)
    out = sc.render_soft(frame, 1, 777, want_float=True)
    assert out["stream_end"] == 777
    assert np.array_equal(out["fimg"].view(np.uint32), sc.render_image(frame)["fimg"].view(np.uint32))
    sc.close()


def test_soft_shadows_stream_window_and_outputs(rtlib, ctx):
    """Frames chained through stream_end; the same frame again (its slice
    already on the device) and device outputs give the same bits; bad
    arguments are refused."""
    torch = pytest.importorskip("torch")
    from raptor_gb300 import scenes
    scene, frame = scenes.icosphere_scene(freq=16, res=128)
    frame = dict(frame, lights=[dict(frame["lights"][0], r=0.7),
                                dict(scenes.spot_light((2.0, 4.0, 2.0), (-0.4, -0.8, -0.4), 0.2, 0.5), r=0.5)])
    sc = rtlib.Scene(ctx, scene)
    a = sc.render_soft(frame, 16, 0)
    b = sc.render_soft(frame, 16, a["stream_end"])
    assert b["stream_end"] - a["stream_end"] == a["stream_end"]
    assert not np.array_equal(a["rgb"], b["rgb"])          # new random points
    again = sc.render_soft(frame, 16, a["stream_end"])
    assert np.array_equal(again["rgb"], b["rgb"])
    dev = torch.empty((128, 128, 3), dtype=torch.uint8, device="cuda")
    fdev = torch.empty((128, 128, 3), dtype=torch.float32, device="cuda")
    sc.render_soft(frame, 16, 0, rgb=dev, fimg=fdev)
    assert np.array_equal(dev.cpu().numpy(), a["rgb"])
    assert np.array_equal(np.clip(fdev.cpu().numpy(), 0, 255).astype(np.uint8), a["rgb"])
    for bad in ({"samples": 0}, {"samples": 65}, {"offset": -1}):
        with pytest.raises(rtlib.RtError):
            sc.render_soft(frame, bad.get("samples", 16), bad.get("offset", 0))
    with pytest.raises(rtlib.RtError):
        sc.render_soft(dict(frame, material=dict(frame["material"], rf=0.5)), 16, 0)
    with pytest.raises(rtlib.RtError):
        sc.render_soft(dict(frame, lights=[dict(frame["lights"][0], r=-1.0)]), 16, 0)
    sc.close()


def test_soft_shadows_read_ahead_frames(rtlib):
    """Consecutive frames, each starting at the last one's stream_end (whose
    numbers a host thread generated while the last frame rendered), a jump
    past the numbers read ahead and a jump back to an earlier position all
    equal the frames a fresh context renders at the same positions."""
    from raptor_gb300 import scenes
    scene, frame = scenes.icosphere_scene(freq=16, res=96)
    frame = dict(frame, lights=[dict(frame["lights"][0], r=0.7)])
    c1 = rtlib.Context(0)
    sc = rtlib.Scene(c1, scene)
    seen = []
    pos = 0
    for _ in range(4):
        out = sc.render_soft(frame, 8, pos, want_float=True)
        seen.append((pos, out))
        pos = out["stream_end"]
    per_frame = seen[0][1]["stream_end"]
    for p in (pos + 3 * per_frame, seen[1][0], seen[2][0]):
        seen.append((p, sc.render_soft(frame, 8, p, want_float=True)))
    sc.close()
    c1.close()
    c2 = rtlib.Context(0)
    fresh = rtlib.Scene(c2, scene)
    for p, out in seen:
        ref = fresh.render_soft(frame, 8, p, want_float=True)
        assert out["stream_end"] == ref["stream_end"] == p + per_frame
        assert np.array_equal(out["fimg"].view(np.uint32), ref["fimg"].view(np.uint32)), p
    fresh.close()
    c2.close()


def test_triangle_lights_match_oracle_float_frames(rtlib, ctx, oracle):
    """480x270 terrain with two triangle-defined lights beside the sun: a
    quad (two triangles) and a 7-triangle spot-light disk.  With 16 samples
    the quad makes 17 rays (its triangle count divides 16) and the disk 16;
    with 6 the quad makes 7 and so does the disk (the binary32 stride lands
    on all seven triangles).  From a nonzero stream position, the float
    image equals the oracle's bit for bit on every pixel with the same
    primary hit, and the stream positions agree."""
    from raptor_gb300 import scenes
    scene, frame = scenes.terrain_scene(size_pow2=256, xres=480, yres=270)
    scene, quad = scenes.add_area_light(scene, [(400.0, 300.0, 400.0), (560.0, 300.0, 400.0),
                                                (560.0, 320.0, 560.0), (400.0, 320.0, 560.0)], rgb=(255.0, 220.0, 190.0))
    scene, disk = scenes.add_area_light(scene, scenes.regular_polygon((250.0, 280.0, 700.0), 50.0, 9, 0.5),
                                        spot=((0.1, -0.95, -0.2), 0.4, 0.9))
    frame = dict(frame, lights=[quad, disk, frame["lights"][0]])
    assert oracle.area_light_rays(2, 16)[0] == 17 and oracle.area_light_rays(7, 6)[0] == 7
    sc = rtlib.Scene(ctx, scene)
    osc = oracle.OracleScene(scene)
    ids = sc.render(dict(frame, lights=[]), want_ids=True)["ids"]
    for samples, offset in ((16, 4321), (6, 99)):
        out = sc.render_soft(frame, samples, offset, want_float=True)
        assert out["stats"].status == 0
        ref = osc.render_soft(frame, samples, offset, threads=NTHREADS, want_ids=True, want_float=True)
        assert out["stream_end"] == ref["stream_end"]
        hits = int((ids >= 0).sum())
        assert out["stream_end"] - offset == hits * 2 * (oracle.area_light_rays(2, samples)[0] +
                                                          oracle.area_light_rays(7, samples)[0])
        assert out["stats"].secondary_rays == hits * (2 * samples + 1)
        same = ids == ref["ids"]
        exact = (out["fimg"].view(np.uint32) == ref["fimg"].view(np.uint32)).all(-1)
        assert exact[same].mean() == 1.0, (samples, exact[same].mean())
        hard = sc.render_image(frame)["fimg"]
        assert (np.abs(hard - out["fimg"]).max(-1) > 1.0).mean() > 0.01
    sc.close()


def test_triangle_lights_bad_arguments(rtlib, ctx):
    """A triangle-defined light with a radius, a directional one, or a
    triangle index outside the scene is refused."""
    from raptor_gb300 import scenes
    scene, frame = scenes.icosphere_scene(freq=8, res=64)
    scene, quad = scenes.add_area_light(scene, [(-0.9, 2.6, -0.9), (0.9, 2.6, -0.9), (0.9, 2.6, 0.9), (-0.9, 2.6, 0.9)])
    sc = rtlib.Scene(ctx, scene)
    assert sc.render_soft(dict(frame, lights=[quad]), 16, 0)["stats"].status == 0
    for bad in (dict(quad, r=0.5), dict(quad, kind=1), dict(quad, tris=[0, scene["tris"].shape[0]]),
                dict(quad, tris=[-1])):
        with pytest.raises(rtlib.RtError):
            sc.render_soft(dict(frame, lights=[bad]), 16, 0)
    sc.close()


def test_soft_shadows_terrain_full_size(rtlib, ctx, oracle):
    """The headline terrain (2,097,152 triangles, 1920x1080) with a
    spherical light of radius 40 beside the sun, 16 samples: against the
    oracle, pixels within one level on >= 99.9 % and the stream position
    after the frame equal; a clean status word."""
    from raptor_gb300 import scenes
    scene, frame = scenes.terrain_scene()
    frame = dict(frame, lights=[dict(scenes.point_light((300.0, 260.0, 500.0)), r=40.0), frame["lights"][0]])
    sc = rtlib.Scene(ctx, scene)
    out = sc.render_soft(frame, 16, 0)
    assert out["stats"].status == 0
    ref = oracle.OracleScene(scene).render_soft(frame, 16, 0, threads=NTHREADS)
    assert out["stream_end"] == ref["stream_end"]
    within1, exact, maxd = pixel_agreement(out["rgb"], ref["rgb"])
    assert within1 >= PIX_FRAC, (within1, exact, maxd)
    assert exact >= 0.999, exact
    sc.close()
