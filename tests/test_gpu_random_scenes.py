"""Randomised parity sweep: seeded random scenes (triangle soups with light
and transparent flags, spheres, heightfields), random cameras, light mixes and
materials (tables of refracting and reflecting materials indexed per
triangle on odd seeds, corner normals for smooth shading on every fourth);
every frame, hit-id map and a batch of random rays is compared
with the oracle under the parity rules of tests/parity.py."""
import numpy as np
import pytest

from parity import PIX_FRAC, compare_hits, pixel_agreement

pytestmark = pytest.mark.gpu


def random_case(seed):
    from raptor_gb300 import scenes
    rng = np.random.default_rng(1000 + seed)
    kind = seed % 3
    if kind == 0:      # soup
        n = int(rng.integers(50, 3000))
        c = rng.uniform(-4, 4, (n, 3))
        v = (c[:, None, :] + rng.uniform(-1, 1, (n, 3, 3)) * rng.uniform(0.1, 1.5)).reshape(-1, 3)
        t = np.arange(3 * n, dtype=np.int32).reshape(-1, 3)
        flags = np.zeros(n, np.uint32)
        flags[rng.uniform(size=n) < 0.05] |= 1
        flags[rng.uniform(size=n) < 0.05] |= 2
        scene = scenes._pack(v, t, rng.uniform(0, 1, (v.shape[0], 3)), flags)
    elif kind == 1:    # sphere, possibly squashed
        v, t = scenes.geodesic_sphere(int(rng.integers(2, 14)))
        v = v * rng.uniform(0.5, 2.0, 3)
        scene = scenes._pack(v, t, rng.uniform(0, 1, (v.shape[0], 3)))
    else:              # heightfield
        size = int(2 ** rng.integers(3, 7))
        h = scenes.diamond_square(size, float(rng.uniform(0.3, 0.8)), int(rng.integers(0, 1 << 30)))
        v, t, hs = scenes.heightfield_mesh(h, 8.0, float(rng.uniform(0.5, 4.0)))
        v = v - np.array([4.0, 0.0, 4.0])
        scene = scenes._pack(v, t, scenes.slope_colours(hs, 8.0 / size, 4.0))
    eye = rng.normal(size=3)
    eye = eye / np.linalg.norm(eye) * rng.uniform(6.0, 12.0)
    res = (int(rng.integers(40, 120)), int(rng.integers(30, 90)))
    cam = scenes.look_at_camera(eye, rng.normal(0, 0.5, 3), float(rng.uniform(30, 80)), res[0], res[1],
                                background=tuple(float(x) for x in rng.uniform(0, 255, 3)))
    lights = []
    for _ in range(int(rng.integers(0, 4))):
        rgb = tuple(float(x) for x in rng.uniform(20, 255, 3))
        if rng.uniform() < 0.5:
            lights.append(scenes.point_light(rng.normal(0, 6, 3), rgb=rgb, d=float(rng.uniform(0, 0.1))))
        else:
            lights.append(scenes.directional_light(rng.normal(size=3), rgb=rgb))
    mat = {"ka": tuple(float(x) for x in rng.uniform(0, 60, 3)), "kd": tuple(float(x) for x in rng.uniform(0, 255, 3)),
           "ks": tuple(float(x) for x in rng.uniform(0, 255, 3)), "ns": float(rng.uniform(1, 60)),
           "rf": float(rng.choice([0.0, 0.0, 0.3, 0.6]))}
    frame = {"camera": cam, "lights": lights, "material": mat}
    if seed % 2 == 1:
        # a table of 1-4 materials, some refracting, indexed per triangle
        table = []
        for _ in range(int(rng.integers(1, 5))):
            table.append(dict(mat, kd=tuple(float(x) for x in rng.uniform(0, 255, 3)),
                              rf=float(rng.choice([0.0, 0.3, 0.6])), tran=float(rng.choice([0.0, 0.4, 0.7])),
                              ri=float(rng.uniform(0.8, 2.2)), flags=int(rng.integers(0, 2))))
        scene["mat_of_tri"] = rng.integers(0, len(table), scene["tris"].shape[0]).astype(np.int32)
        frame["materials"] = table
        # shadow rays pass the triangles of refracting materials (the
        # reference's material::is_transparent, set when tran > 0)
        see_through = np.array([m["tran"] > 0.0 for m in table])[scene["mat_of_tri"]]
        scene["flags"] = (scene["flags"] & np.uint32(1)) | np.where(see_through, np.uint32(2), np.uint32(0))
    if seed % 4 == 2:
        # smooth shading: unit corner normals near the face normal, some
        # triangles without (first float FLT_MAX)
        nt = scene["tris"].shape[0]
        cn = rng.normal(size=(nt, 3, 3)).astype(np.float32)
        cn /= np.linalg.norm(cn, axis=2, keepdims=True)
        cn = cn.reshape(nt, 9)
        cn[rng.uniform(size=nt) < 0.2, 0] = np.float32(3.4028234663852886e38)
        scene["corner_normals"] = cn
    return scene, frame, rng


@pytest.mark.parametrize("seed", range(24))
def test_random_scene_vs_oracle(rtlib, ctx, oracle, seed):
    scene, frame, rng = random_case(seed)
    sc = rtlib.Scene(ctx, scene)
    osc = oracle.OracleScene(scene)
    # random rays: closest and any hit
    v = scene["verts"].astype(np.float64)
    o = rng.uniform(v.min(0) - 2, v.max(0) + 2, (4000, 3)).astype(np.float32)
    d = rng.normal(size=(4000, 3))
    d = (d / np.linalg.norm(d, axis=1)[:, None]).astype(np.float32)
    tmax = rng.uniform(0.5, 15.0, 4000).astype(np.float32)
    h = sc.closest(rtlib.rays_array(o, d))
    rid, rt_, _, _ = osc.closest(o, d)
    mismatch, _ = compare_hits(scene["verts"], scene["tris"], o, d, h["tri"], h["t"], rid, rt_)
    assert not mismatch.any(), np.nonzero(mismatch)[0][:8]
    occ = sc.any(rtlib.rays_array(o, d, tmax=tmax))
    rocc = osc.any(o, d, tmax)
    # occlusion: exact except rays whose nearest qualifying hit is at tmax or EPSILON (within 1e-5) or near an edge
    differ = occ.astype(bool) != rocc.astype(bool)
    assert differ.mean() < 2e-3, differ.mean()
    # frame
    got = sc.render(frame, want_ids=True)
    want = osc.render(frame, want_ids=True)
    within1, exact, worst = pixel_agreement(got["rgb"], want["rgb"])
    assert within1 >= 0.995 and exact >= 0.99, (within1, exact, worst)
    same_id = (got["ids"] == want["ids"]).mean()
    assert same_id >= 0.995, same_id
    sc.close()
