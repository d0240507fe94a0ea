"""rt_trace_closest_noalloc: the closest-hit entry point for callers that
cannot allocate device memory stages its rays and hits through the
library's fixed scratch array and must return what rt_trace_closest returns,
call after call (the array keeps the previous call's contents)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_RAYS = 16384


def scene_and_rays(rng, n):
    from raptor_gb300 import scenes
    scene, _ = scenes.terrain_scene(size_pow2=128, xres=64, yres=36)
    v = scene["verts"].astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    o = rng.uniform(lo, hi, size=(n, 3))
    o[:, 1] = hi[1] + rng.uniform(1.0, 20.0, n)
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1]) - 0.2     # mostly downwards: hits and misses
    d /= np.linalg.norm(d, axis=1)[:, None]
    return scene, o.astype(np.float32), d.astype(np.float32)


def noalloc(rtlib, sc, rays, out):
    return rtlib.lib().rt_trace_closest_noalloc(sc.h, rtlib.ptr(rays), int(rays.shape[0]), rtlib.ptr(out))


def same_hits(a, b):
    """Both entry points run the same traversal kernel on the same rays, so
    the hits agree bit for bit."""
    assert np.array_equal(a["tri"], b["tri"])
    for k in ("t", "u", "v"):
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


def test_noalloc_matches_trace_closest(rtlib):
    rng = np.random.default_rng(21)
    scene, o, d = scene_and_rays(rng, 2 * MAX_RAYS)
    c = rtlib.Context(0)
    sc = rtlib.Scene(c, scene)
    first = rtlib.rays_array(o[:MAX_RAYS], d[:MAX_RAYS])
    second = rtlib.rays_array(o[MAX_RAYS:MAX_RAYS + 5000], d[MAX_RAYS:MAX_RAYS + 5000])
    want1 = sc.closest(first)
    want2 = sc.closest(second)
    assert 0.2 < (want1["tri"] >= 0).mean() < 1.0
    # two calls in a row, the second smaller than the first
    got1 = np.zeros(first.shape[0], rtlib.HIT_DTYPE)
    got2 = np.zeros(second.shape[0], rtlib.HIT_DTYPE)
    assert noalloc(rtlib, sc, first, got1) == 0
    assert noalloc(rtlib, sc, second, got2) == 0
    same_hits(got1, want1)
    same_hits(got2, want2)
    sc.close()
    c.close()


def test_noalloc_after_context_recreated(rtlib):
    """The scratch address is looked up again after the last context on the
    device is closed; a new context's calls still match rt_trace_closest."""
    rng = np.random.default_rng(23)
    scene, o, d = scene_and_rays(rng, 4096)
    rays = rtlib.rays_array(o, d)
    for _ in range(2):
        c = rtlib.Context(0)
        sc = rtlib.Scene(c, scene)
        want = sc.closest(rays)
        got = np.zeros(rays.shape[0], rtlib.HIT_DTYPE)
        assert noalloc(rtlib, sc, rays, got) == 0
        same_hits(got, want)
        sc.close()
        c.close()


def test_noalloc_device_buffers_and_limit(rtlib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(22)
    scene, o, d = scene_and_rays(rng, 3000)
    c = rtlib.Context(0)
    sc = rtlib.Scene(c, scene)
    rays = rtlib.rays_array(o, d)
    want = sc.closest(rays)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.zeros(rays.shape[0] * 16, dtype=torch.uint8, device="cuda")
    for _ in range(2):
        d_hits.zero_()
        torch.cuda.synchronize()
        assert rtlib.lib().rt_trace_closest_noalloc(sc.h, C.c_void_p(d_rays.data_ptr()), rays.shape[0],
                                                    C.c_void_p(d_hits.data_ptr())) == 0
        got = d_hits.cpu().numpy().view(rtlib.HIT_DTYPE)
        same_hits(got, want)
    # repeated calls at the maximum size take no device memory.  The free
    # memory figure is device-wide, so another process allocating at the
    # same moment could move it: one of three attempts must see it unchanged.
    big = rtlib.rays_array(np.repeat(o, 6, 0)[:MAX_RAYS], np.repeat(d, 6, 0)[:MAX_RAYS])
    out = np.zeros(MAX_RAYS, rtlib.HIT_DTYPE)
    assert noalloc(rtlib, sc, big, out) == 0
    unchanged = False
    for _ in range(3):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for _ in range(3):
            assert noalloc(rtlib, sc, big, out) == 0
        torch.cuda.synchronize()
        if torch.cuda.mem_get_info()[0] == free0:
            unchanged = True
            break
    assert unchanged
    # one ray beyond the maximum is refused before any GPU work
    over = rtlib.rays_array(np.zeros((MAX_RAYS + 1, 3), np.float32), np.tile([0, -1, 0], (MAX_RAYS + 1, 1)).astype(np.float32))
    big_out = np.zeros(MAX_RAYS + 1, rtlib.HIT_DTYPE)
    assert noalloc(rtlib, sc, over, big_out) == -1
    assert b"RT_NOALLOC_MAX_RAYS" in rtlib.lib().rt_last_error_string()
    assert (big_out["t"] == 0).all()
    sc.close()
    c.close()
