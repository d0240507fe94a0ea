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
