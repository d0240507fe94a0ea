"""Distributed ray tracing (rt_render_distributed): the reference's ray tree
with SOFT_SHADOW and DIFFUSE_REFLECTIONS.

Reference-stream frames (mirror and glass trees with soft shadows at every
hit) against the reference's own frames (tests/golden/ref_distributed.npz,
from the SOFT_SHADOW = 16 build) and the oracle's restatement; per-pixel-
stream frames (diffuse reflections and refractions) against the oracle
drawing the same per-pixel streams (oracle/rtoracle.c,
ro_render_distributed).  Frames are compared pixel for pixel: equal except
where the camera ray passes within 1e-5 of a triangle edge (ties), and the
numbers drawn equal."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from parity import edge_distance

pytestmark = pytest.mark.gpu

NTHREADS = max(1, os.cpu_count() or 1)


@pytest.fixture(scope="module")
def dist_golden():
    return np.load(os.path.join(GOLDEN, "ref_distributed.npz"))


def golden_cases(g):
    k = 0
    while f"dist{k}_rgb" in g.files:
        frame = json.loads(g[f"dist{k}_frame"].tobytes().decode())
        scene = {key: g[f"dist{k}_{key}"] for key in ("verts", "tris", "vattr", "flags", "mat_of_tri")
                 if f"dist{k}_{key}" in g.files}
        yield k, scene, frame, int(g[f"dist{k}_diffuse"][0]), int(g[f"dist{k}_offset"][0]), g[f"dist{k}_rgb"]
        k += 1


def edge_pixels(oracle, scene, frame, ids):
    o, d = oracle.camera_rays(frame["camera"])
    H, W = frame["camera"]["yres"], frame["camera"]["xres"]
    return (edge_distance(scene["verts"], scene["tris"], ids.reshape(-1), o, d) < 1e-5).reshape(H, W)


def test_distributed_match_reference(rtlib, ctx, oracle, dist_golden):
    """The reference's frames of the SOFT_SHADOW = 16 build (glass and
    mirror trees; spherical, spot and triangle-defined lights), each from
    the stream position the reference had reached: every pixel equal but
    edge ties, and the stream position after each frame the reference's.
    The DIFFUSE_REFLECTIONS frames are refused on the reference's stream."""
    soft = int(dist_golden["soft"][0])
    cases = list(golden_cases(dist_golden))
    for n, (k, scene, frame, diffuse, offset, ref) in enumerate(cases):
        sc = rtlib.Scene(ctx, scene)
        if diffuse:
            with pytest.raises(rtlib.RtError):
                sc.render_distributed(frame, soft=soft, diffuse=diffuse, offset=offset)
            sc.close()
            continue
        out = sc.render_distributed(frame, soft=soft, offset=offset)
        assert out["stats"].status == 0
        nxt = [c for c in cases[n + 1:] if c[3] == 0]
        expect_end = nxt[0][4] if nxt else int(dist_golden["stream_end"][0])
        assert out["stream_end"] == expect_end, (k, out["stream_end"], expect_end)
        ids = sc.render(dict(frame, lights=[]), want_ids=True)["ids"]
        diff = np.abs(out["rgb"].astype(int) - ref.astype(int)).max(-1) > 0
        near = edge_pixels(oracle, scene, frame, ids)
        assert not (diff & ~near).any(), (k, np.argwhere(diff & ~near)[:5])
        sc.close()


def test_distributed_reference_stream_matches_oracle(rtlib, ctx, oracle):
    """256x256 glass scene (refraction and reflection trees), a spherical
    light of radius 0.7 and a directional light, 16 soft samples, from
    stream position 777: the float image equals the oracle's bit for bit on
    every pixel with the same primary hit, and the stream positions agree.
    The frame's second render reuses the slice already on the device."""
    from raptor_gb300 import scenes
    scene, frame = scenes.glass_scene(freq=16, res=256)
    frame = dict(frame, lights=[dict(frame["lights"][0], r=0.7), frame["lights"][1]])
    sc = rtlib.Scene(ctx, scene)
    out = sc.render_distributed(frame, soft=16, offset=777, want_float=True)
    assert out["stats"].status == 0
    ref = oracle.OracleScene(scene).render_distributed(frame, soft=16, offset=777, want_ids=True, want_float=True)
    assert out["stream_end"] == 777 + ref["drawn"]
    ids = sc.render(dict(frame, lights=[]), want_ids=True)["ids"]
    same = ids == ref["ids"]
    exact = (out["fimg"].view(np.uint32) == ref["fimg"].view(np.uint32)).all(-1)
    assert exact[same].mean() > 0.9995, exact[same].mean()
    again = sc.render_distributed(frame, soft=16, offset=777, want_float=True)
    assert np.array_equal(again["fimg"].view(np.uint32), out["fimg"].view(np.uint32))
    sc.close()


@pytest.mark.parametrize("case", [3, 4])
def test_distributed_pixel_streams_match_oracle(rtlib, ctx, oracle, dist_golden, case):
    """The diffuse fixtures' scenes (diffuse reflections and refractions of
    16 rays, 16 soft samples, triangle-defined and spot lights) on per-pixel
    streams: the float image equals the oracle's drawing the same streams,
    bit for bit on every pixel with the same primary hit; the numbers drawn
    agree."""
    k, scene, frame, diffuse, _, _ = list(golden_cases(dist_golden))[case]
    assert diffuse > 0
    sc = rtlib.Scene(ctx, scene)
    out = sc.render_distributed(frame, soft=16, diffuse=diffuse, stream=rtlib.RT_STREAM_PIXEL, seed=2024,
                                want_float=True)
    assert out["stats"].status == 0
    ref = oracle.OracleScene(scene).render_distributed(frame, soft=16, diffuse=diffuse, stream=oracle.STREAM_PIXEL,
                                                       seed=2024, threads=NTHREADS, want_ids=True, want_float=True)
    ids = sc.render(dict(frame, lights=[]), want_ids=True)["ids"]
    same = ids == ref["ids"]
    exact = (out["fimg"].view(np.uint32) == ref["fimg"].view(np.uint32)).all(-1)
    assert exact[same].mean() > 0.999, exact[same].mean()
    assert abs(out["stream_end"] - ref["drawn"]) <= 0.001 * ref["drawn"]
    # the diffuse rays did something: another seed gives another frame
    other = sc.render_distributed(frame, soft=16, diffuse=diffuse, stream=rtlib.RT_STREAM_PIXEL, seed=2025)
    assert not np.array_equal(other["rgb"], out["rgb"])
    sc.close()


def test_distributed_without_trees_is_the_soft_shadow_frame(rtlib, ctx):
    """No mirror or glass: the reference-stream frame is rt_render_soft_shadows'
    frame; on per-pixel streams, the same frame twice is identical."""
    from raptor_gb300 import scenes
    scene, frame = scenes.icosphere_scene(freq=16, res=128)
    frame = dict(frame, lights=[dict(frame["lights"][0], r=0.7)])
    sc = rtlib.Scene(ctx, scene)
    a = sc.render_distributed(frame, soft=16, offset=5, want_float=True)
    b = sc.render_soft(frame, 16, 5, want_float=True)
    assert a["stream_end"] == b["stream_end"]
    assert np.array_equal(a["fimg"].view(np.uint32), b["fimg"].view(np.uint32))
    p1 = sc.render_distributed(frame, soft=16, stream=rtlib.RT_STREAM_PIXEL, seed=3, want_float=True)
    p2 = sc.render_distributed(frame, soft=16, stream=rtlib.RT_STREAM_PIXEL, seed=3, want_float=True)
    assert np.array_equal(p1["fimg"].view(np.uint32), p2["fimg"].view(np.uint32))
    hits = int(p1["stats"].primary_hits)
    assert p1["stream_end"] == hits * 3 * 16
    sc.close()


def test_distributed_bad_arguments(rtlib, ctx):
    """Sample counts, stream kind, diffuse rays on the reference's stream,
    and trees past RT_MAX_TREE_RAYS are refused."""
    from raptor_gb300 import scenes
    scene, frame = scenes.glass_scene(freq=8, res=32)
    sc = rtlib.Scene(ctx, scene)
    diffuse_mats = [dict(frame["materials"][0], rfd=0.2), frame["materials"][1]]
    fd = dict(frame, materials=diffuse_mats)
    assert sc.render_distributed(fd, soft=4, diffuse=4, stream=rtlib.RT_STREAM_PIXEL)["stats"].status == 0
    for kw in ({"soft": 0}, {"soft": 65}, {"diffuse": -1}, {"diffuse": 65}, {"stream": 2}):
        with pytest.raises(rtlib.RtError):
            sc.render_distributed(frame, **kw)
    with pytest.raises(rtlib.RtError):
        sc.render_distributed(fd, soft=4, diffuse=4, stream=rtlib.RT_STREAM_REFERENCE)
    big = [dict(frame["materials"][0], rf=0.9, rfd=0.2), frame["materials"][1]]
    with pytest.raises(rtlib.RtError):
        sc.render_distributed(dict(frame, materials=big), soft=4, diffuse=64, stream=rtlib.RT_STREAM_PIXEL)
    sc.close()
