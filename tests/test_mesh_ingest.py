"""Scene ingest (rt_mesh_parse / rt_mesh_load): OFF and PLY files give the
triangles the reference's own parsers put into its primitive_store, in the
same order and bit for bit (tests/golden: synthetic files with convex and
concave polygons, collinear vertices, a star, degenerate triangles, CRLF
line ends, comments, vertex normals and colours, face intensity and face
colours, big-endian binary, OBJ index forms v, v/t, v//n, v/t/n with
negative indices, usemtl groups), so triangle ids match the reference's."""
import numpy as np
import pytest

from conftest import GOLDEN


def mesh_cases():
    import os
    g = np.load(os.path.join(GOLDEN, "ref_small.npz"))
    k = 0
    out = []
    while f"mesh{k}_bytes" in g.files:
        out.append(k)
        k += 1
    return out


@pytest.mark.parametrize("k", mesh_cases())
def test_mesh_matches_reference_parser(rtlib, golden_npz, k):
    data = golden_npz[f"mesh{k}_bytes"].tobytes()
    kind = int(golden_npz[f"mesh{k}_kind"][0])
    want = golden_npz[f"mesh{k}_tris"]
    m = rtlib.parse_mesh(data, kind)
    got = m["verts"][m["tris"]].reshape(-1, 9)
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert m["kd"] == ((170.0,) * 3 if kind == 1 else (200.0,) * 3)
    nmat = int(golden_npz[f"mesh{k}_nmat"][0])
    if m["tri_rgb"] is not None:
        # one material per distinct face colour, plus the default one
        assert len({tuple(c) for c in m["tri_rgb"]}) + 1 == nmat
    elif m["tri_mat"] is not None:
        # OBJ: the default material plus one per distinct usemtl name
        assert m["nmat"] == nmat and set(np.unique(m["tri_mat"])) <= set(range(nmat))
    else:
        assert nmat == 1


def test_obj_material_groups(rtlib, golden_npz):
    """usemtl switches the material of the triangles that follow; names
    repeat onto their first index."""
    k = next(i for i in mesh_cases() if int(golden_npz[f"mesh{i}_kind"][0]) == 3)
    text = golden_npz[f"mesh{k}_bytes"].tobytes().decode()
    m = rtlib.parse_mesh(text.encode(), rtlib.RT_MESH_OBJ)
    # the first usemtl precedes the first face: no triangle keeps material 0
    assert m["tri_mat"].min() == 1 and m["nmat"] == 4
    names = []
    for line in text.splitlines():
        if line.startswith("usemtl "):
            names.append(line.split()[1])
    assert list(dict.fromkeys(names)) == ["stone", "glass", "metal"]


def test_mesh_load_from_file_and_errors(rtlib, golden_npz, tmp_path):
    data = golden_npz["mesh0_bytes"].tobytes()
    p = tmp_path / "scene.off"
    p.write_bytes(data)
    a = rtlib.load_mesh(p)
    b = rtlib.parse_mesh(data, rtlib.RT_MESH_OFF)
    assert np.array_equal(a["verts"], b["verts"]) and np.array_equal(a["tris"], b["tris"])
    for bad in (b"OFX\n3 1 0\n", b"OFF\n3 1 0\n0 0 0\n1 0 0\n0 1 0\n3 0 1 7\n", b"ply\nformat binary_little_endian 1.0\n"):
        with pytest.raises(rtlib.RtError):
            rtlib.parse_mesh(bad, rtlib.RT_MESH_OFF if bad.startswith(b"OF") else rtlib.RT_MESH_PLY)
    with pytest.raises(rtlib.RtError):
        rtlib.load_mesh(tmp_path / "missing.off")
    with pytest.raises(rtlib.RtError):
        rtlib.load_mesh(tmp_path / "scene.xyz")


def mesh_scene(rtlib, golden_npz, k):
    """The parsed mesh as a scene with the reference parser's materials
    (phong_shader: ka 0, ks 0, kd the default or the face colour) and the
    frame the reference rendered it with."""
    import json
    data = golden_npz[f"mesh{k}_bytes"].tobytes()
    kind = int(golden_npz[f"mesh{k}_kind"][0])
    m = rtlib.parse_mesh(data, kind)
    base = {"ka": (0.0, 0.0, 0.0), "kd": tuple(m["kd"]), "ks": (0.0, 0.0, 0.0), "ns": 0.0, "flags": 1}
    scene = {"verts": m["verts"], "tris": m["tris"], "vattr": None, "flags": None,
             "corner_normals": m["corner_normals"]}
    table = [base]
    if m["tri_rgb"] is not None:
        colours = sorted({tuple(int(x) for x in c) for c in m["tri_rgb"]})
        table += [dict(base, kd=tuple(float(x) for x in c)) for c in colours]
        index = {c: i + 1 for i, c in enumerate(colours)}
        scene["mat_of_tri"] = np.array([index[tuple(int(x) for x in c)] for c in m["tri_rgb"]], np.int32)
    frame = json.loads(golden_npz[f"mesh{k}_frame"].tobytes().decode())
    frame["materials"] = table
    frame["material"] = base
    return scene, frame, golden_npz[f"mesh{k}_render_rgb"]


@pytest.mark.parametrize("k", mesh_cases())
def test_ingested_scene_renders_as_reference(rtlib, oracle, golden_npz, k):
    """Parse -> render: the restatement renders the loaded mesh with the
    parser's materials to the reference's own frame of the same file
    (parser + bvh + ray_tracer), pixel for pixel but for tie pixels."""
    from parity import pixel_agreement
    scene, frame, ref = mesh_scene(rtlib, golden_npz, k)
    out = oracle.OracleScene(scene).render(frame)["rgb"]
    within1, exact, _ = pixel_agreement(out, ref)
    assert exact >= 0.995, exact
