"""Batched persistent renderer: many scenes, resolutions and ray mixes in
one graph-captured launch must give exactly the frames of the single-frame
path (rt_render / rt_render_ao), whatever launch shape the autotuner picks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_batch(n=10, seed=11):
    from raptor_gb300 import scenes
    return scenes.batched_scenes(n=n, seed=seed, tri_lo=200, tri_hi=20000)


def shrink(frame, cap=256):
    """Cap resolutions so the test stays small (keeps aspect, odd sizes kept
    to exercise partial tiles)."""
    cam = dict(frame["camera"])
    s = max(cam["xres"], cam["yres"]) / cap
    if s > 1:
        cam["xres"] = int(cam["xres"] / s) + 1
        cam["yres"] = int(cam["yres"] / s) + 1
    f = dict(frame)
    f["camera"] = cam
    return f


@pytest.fixture(scope="module")
def batch_setup(rtlib, ctx):
    torch = pytest.importorskip("torch")
    items = [(sc, shrink(fr)) for sc, fr in small_batch()]
    b = rtlib.Batch(ctx)
    idx = [b.add_scene(sc) for sc, _ in items]
    # an empty scene in the middle of the batch: every ray misses
    empty = {"verts": np.zeros((0, 3), np.float32), "tris": np.zeros((0, 3), np.int32)}
    e_idx = b.add_scene(empty)
    b.build()
    bufs, jobs = [], []
    for i, (sc, fr) in enumerate(items):
        W, H = fr["camera"]["xres"], fr["camera"]["yres"]
        rgb = torch.zeros((H, W, 3), dtype=torch.uint8, device="cuda")
        ids = torch.zeros((H, W), dtype=torch.int32, device="cuda")
        bufs.append((rgb, ids))
        jobs.append(rtlib.make_job(idx[i], fr, rgb, ids))
    fr0 = items[0][1]
    erg = torch.zeros((fr0["camera"]["yres"], fr0["camera"]["xres"], 3), dtype=torch.uint8, device="cuda")
    eid = torch.zeros(erg.shape[:2], dtype=torch.int32, device="cuda")
    jobs.append(rtlib.make_job(e_idx, fr0, erg, eid))
    b.set_jobs(jobs)
    return b, items, bufs, (erg, eid, fr0), torch


def plain_frames(rtlib, ctx, items):
    out = []
    for sc, fr in items:
        s = rtlib.Scene(ctx, sc)
        r = s.render(fr, want_ids=True)
        out.append((r["rgb"].copy(), r["ids"].copy(), r["stats"]))
        s.close()
    return out


def test_batched_equals_plain(rtlib, ctx, batch_setup):
    b, items, bufs, empty, torch = batch_setup
    assert any(fr.get("ao") for _, fr in items) and any(not fr.get("ao") for _, fr in items)
    st = b.render()
    plain = plain_frames(rtlib, ctx, items)
    prim = sec = 0
    for (rgb, ids), (prgb, pids, pst) in zip(bufs, plain):
        assert np.array_equal(rgb.cpu().numpy(), prgb)
        assert np.array_equal(ids.cpu().numpy(), pids)
        prim += pst.primary_rays
        sec += pst.secondary_rays
    erg, eid, fr0 = empty
    npx = fr0["camera"]["xres"] * fr0["camera"]["yres"]
    assert st.primary_rays == prim + npx
    assert st.secondary_rays == sec
    assert (eid.cpu().numpy() == -1).all()
    bg = np.array(fr0["camera"]["background"], np.float32)
    assert (erg.cpu().numpy() == np.clip(bg, 0, 255).astype(np.uint8)).all()


def test_autotune_keeps_results(rtlib, ctx, batch_setup):
    b, items, bufs, _, torch = batch_setup
    b.render()
    before = [rgb.cpu().numpy().copy() for rgb, _ in bufs]
    best = b.autotune(reps=1)
    assert best["block_threads"] in (64, 128, 256) and best["tile_w"] in (8, 16) and best["ms"] > 0
    for rgb, _ in bufs:
        rgb.zero_()
    b.render()
    for (rgb, _), ref in zip(bufs, before):
        assert np.array_equal(rgb.cpu().numpy(), ref)
    assert best["stack_entries"] in (16, 24, 48)
    # every shape gives the same frames
    for shape in ((64, 4, 16, 1, 48), (256, 2, 8, 1, 16), (128, 1, 8, 1, 24), (64, 1, 16, 0, 48),
                  (256, 1, 8, 0, 48)):
        b.set_config(*shape)
        b.render()
        for (rgb, _), ref in zip(bufs, before):
            assert np.array_equal(rgb.cpu().numpy(), ref)


def test_batch_rejects_host_outputs(rtlib, ctx):
    from raptor_gb300 import scenes
    sc, fr = scenes.icosphere_scene(freq=4, res=32)
    b = rtlib.Batch(ctx)
    i = b.add_scene(sc)
    b.build()
    host = np.zeros((32, 32, 3), np.uint8)
    with pytest.raises(rtlib.RtError):
        b.set_jobs([rtlib.make_job(i, fr, host)])
