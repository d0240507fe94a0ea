"""The bilateral tone mapper (RT_TONE_GLOBAL_BILATERAL,
camera::bilateral_filter_tone_map, camera.cc:1632-1812) on the GPU: against
the reference's own frames (tests/golden/ref_bilateral.npz, written by the
reference with its FFTW calls served by double-precision transforms) and
against the oracle's restatement.  The Gaussian blur is computed exactly
here, so FFTW's single-precision rounding is all that separates the frames:
one level at most, on a small fraction of pixels."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def cases():
    g = np.load(os.path.join(GOLDEN, "ref_bilateral.npz"))
    k = 0
    while f"bil{k}_rgb" in g.files:
        yield k, g[f"bil{k}_fimg"], json.loads(g[f"bil{k}_args"].tobytes().decode()), g[f"bil{k}_rgb"]
        k += 1


def test_bilateral_tone_map_matches_reference(rtlib, ctx, oracle):
    """Four fixed float frames (terrain, glass sphere; gamma, 2x2
    anti-aliasing, contrast stretch): the GPU frame within one level of the
    reference's on every pixel and equal on >= 99.9 %; within one level of
    the oracle's too."""
    n = 0
    for k, fimg, args, ref in cases():
        aa = tuple(args["aa"])
        got = ctx.tone_map_image(fimg, args["camera"], args["tone"], aa)
        d = np.abs(got.astype(int) - ref.astype(int)).max(-1)
        assert d.max() <= 1, (args["name"], d.max())
        assert (d == 0).mean() >= 0.999, (args["name"], (d == 0).mean())
        mine = oracle.downsample_rgb8(oracle.tone_map_frame(fimg, args["tone"], args["camera"]), *aa)
        assert np.abs(got.astype(int) - mine.astype(int)).max() <= 1
        n += 1
    assert n == 4


def test_bilateral_render_tone_mapped_vs_oracle(rtlib, ctx, oracle):
    """A rendered frame tone mapped on the GPU (rt_render_tone_mapped with
    the bilateral mode) against the oracle's render and restatement: dim
    lights keep the frame's contrast; within one level on every pixel."""
    from raptor_gb300 import scenes
    scene, frame = scenes.glass_scene(freq=16, res=200)
    # a colour is light x (kd, ks) + ka: dimming the lights, ka and the sky
    # by 300 dims the frame by 300
    frame = dict(frame, lights=[dict(l, rgb=tuple(c / 300.0 for c in l["rgb"])) for l in frame["lights"]],
                 camera=dict(frame["camera"], background=tuple(c / 300.0 for c in frame["camera"]["background"])),
                 materials=[dict(m, ka=tuple(c / 300.0 for c in m["ka"])) for m in frame["materials"]])
    tone = {"mode": 8, "gamma": 2.2}
    sc = rtlib.Scene(ctx, scene)
    got = sc.render_tone_mapped(frame, tone)["rgb"]
    osc = oracle.OracleScene(scene)
    want = oracle.render_tone_mapped(osc, frame, tone)
    assert got.std() > 10.0
    assert np.abs(got.astype(int) - want.astype(int)).max() <= 1
    sc.close()


def test_bilateral_grid_limit(rtlib, ctx):
    """A frame whose grid would pass 2^26 cells is refused."""
    fimg = np.full((8, 20000, 3), 10.0, np.float32)
    cam = {"pos": (0.0, 0.0, 0.0), "x_axis": (1.0, 0.0, 0.0), "y_axis": (0.0, 1.0, 0.0), "z_axis": (0.0, 0.0, 1.0),
           "background": (0.0, 0.0, 0.0), "w": 1.0, "h": 1.0, "t": 1.0, "xres": 20000, "yres": 8}
    with pytest.raises(rtlib.RtError):
        ctx.tone_map_image(fimg, cam, {"mode": 8})
