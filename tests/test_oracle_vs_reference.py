"""The C restatement against the reference itself at FULL benchmark size:
the reference's own bvh + ray_tracer() + clip_image_to_rgb (compiled from
its sources by oracle/refbuild/Makefile) on the icosphere 512^2 and terrain
1920x1080 frames.  Runs where the reference harness was built (x86-64 with
the reference tree present); skipped elsewhere."""
import os

import numpy as np
import pytest

from parity import PIX_FRAC, compare_hits, pixel_agreement


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available():
        pytest.skip("reference harness not built on this host")
    return oracle


@pytest.mark.parametrize("workload", ["icosphere", "terrain"])
def test_full_frame_restatement_equals_reference(ref, workload):
    from raptor_gb300 import scenes
    scene, frame = scenes.icosphere_scene() if workload == "icosphere" else scenes.terrain_scene()
    rs = ref.RefScene(scene, frame["material"])
    rr = rs.render(frame)
    osc = ref.OracleScene(scene)
    ro = osc.render(frame, threads=os.cpu_count() or 1, want_ids=True)
    within1, exact, _ = pixel_agreement(ro["rgb"], rr["rgb"])
    assert exact >= 0.9999 and within1 >= PIX_FRAC, (exact, within1)
    # primary hits of the reference's own traversal on the reference's camera rays
    og, dr = ref.camera_rays(frame["camera"], lib=ref.ref_lib())
    step = 7 if workload == "terrain" else 1
    og, dr = og[::step], dr[::step]
    rid, rt, _, _ = rs.closest(og, dr)
    oid, ot, _, _ = osc.closest(og, dr)
    mismatch, excluded = compare_hits(scene["verts"], scene["tris"], og, dr, oid, ot, rid, rt)
    assert not mismatch.any()
    same = oid == rid
    assert np.array_equal(ot[same].view(np.uint32), rt[same].view(np.uint32))


@pytest.mark.parametrize("seed", range(1, 24, 2))
def test_random_material_tables_equal_reference(ref, seed):
    """The randomised scenes with per-triangle material tables (reflecting
    and refracting entries): the restatement's frame equals the reference's
    on every pixel."""
    from test_gpu_random_scenes import random_case
    scene, frame, _ = random_case(seed)
    rr = ref.RefScene(scene, frame["materials"]).render(frame)
    ro = ref.OracleScene(scene).render(frame)
    within1, exact, _ = pixel_agreement(ro["rgb"], rr["rgb"])
    assert exact == 1.0, (exact, within1)


def random_polygon_off(seed, nfaces=1500):
    """An OFF file of random planar polygons in random orientations: star-
    shaped and spiky (concave) rings of 3..14 vertices, some with repeated
    or collinear vertices."""
    rng = np.random.default_rng(seed)
    verts, faces = [], []
    for _ in range(nfaces):
        n = int(rng.integers(3, 15))
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        r = rng.uniform(0.2, 1.5, n) if rng.uniform() < 0.6 else np.ones(n)
        pts = np.stack([np.cos(ang) * r, np.sin(ang) * r, np.zeros(n)], 1)
        if rng.uniform() < 0.1 and n > 3:
            pts[1] = 0.5 * (pts[0] + pts[2])          # a collinear middle vertex
        q = np.linalg.qr(rng.normal(size=(3, 3)))[0]
        pts = pts @ q.T + rng.uniform(-20, 20, 3)
        base = len(verts)
        verts.extend(pts.astype(np.float32).tolist())
        faces.append(list(range(base, base + n)))
    lines = ["OFF", f"{len(verts)} {len(faces)} 0"]
    lines += [" ".join(repr(float(np.float32(c))) for c in v) for v in verts]
    lines += [" ".join([str(len(f))] + [str(i) for i in f]) for f in faces]
    return ("\n".join(lines) + "\n").encode()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_polygons_triangulated_as_reference(ref, tmp_path, seed):
    """rt_mesh_parse triangulates random concave polygons exactly as the
    reference's face_to_triangles (polygon_to_triangles.h), triangle by
    triangle."""
    from raptor_gb300 import core
    data = random_polygon_off(seed)
    p = tmp_path / "poly.off"
    p.write_bytes(data)
    want, _ = ref.ref_parse_mesh(p, 1)
    m = core.parse_mesh(data, core.RT_MESH_OFF)
    got = m["verts"][m["tris"]].reshape(-1, 9)
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("seed", [4, 5])
def test_random_polygons_obj_as_reference(ref, tmp_path, seed):
    """The same random polygons as an OBJ file (index forms v, v/t, v//n,
    v/t/n, some negative): rt_mesh_parse matches obj_parser triangle by
    triangle."""
    from raptor_gb300 import core
    rng = np.random.default_rng(seed)
    off = random_polygon_off(seed, nfaces=800).decode().splitlines()
    nv, nf, _ = map(int, off[1].split())
    verts = off[2:2 + nv]
    lines = ["# random polygons"] + [f"v {v}" for v in verts] + [f"vn 0 0 1", "vt 0.5 0.5"]
    for k, f in enumerate(off[2 + nv:2 + nv + nf]):
        idx = [int(x) for x in f.split()[1:]]
        if k % 97 == 0:
            lines.append(f"usemtl m{k % 3}")
        toks = []
        for i in idx:
            vi = str(i + 1) if rng.uniform() < 0.7 else str(i - nv)
            form = int(rng.integers(0, 4))
            toks.append([vi, f"{vi}/1", f"{vi}//1", f"{vi}/-1/1"][form])
        lines.append("f " + " ".join(toks))
    data = ("\n".join(lines) + "\n").encode()
    p = tmp_path / "poly.obj"
    p.write_bytes(data)
    want, nmat = ref.ref_parse_mesh(p, 3)
    m = core.parse_mesh(data, core.RT_MESH_OBJ)
    got = m["verts"][m["tris"]].reshape(-1, 9)
    assert got.shape == want.shape and m["nmat"] == nmat
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
