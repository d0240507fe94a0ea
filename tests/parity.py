"""Parity criteria shared by the tests.

Hit ids must be bit-exact and t within 1e-5 relative, except for rays the
criterion excludes: rays whose hit (on either side) lies within 1e-5 of a
triangle edge in FP64 barycentrics, and exact ties (several triangles at the
same distance; the reference keeps the first one its traversal meets, the
CUDA core the lowest id).  Pixels must be within +-1 LSB on >= 99.9%.
"""
import numpy as np

EDGE_EPS = 1e-5
T_REL = 1e-5
PIX_FRAC = 0.999


def edge_distance(verts, tris, ids, o, d):
    """Smallest FP64 barycentric coordinate of the ray's hit on triangle
    ids[i] (inf where ids[i] < 0)."""
    out = np.full(ids.shape[0], np.inf)
    m = ids >= 0
    if not m.any():
        return out
    t = tris[ids[m]]
    a = verts[t[:, 0]].astype(np.float64)
    b = verts[t[:, 1]].astype(np.float64)
    c = verts[t[:, 2]].astype(np.float64)
    oo = o[m].astype(np.float64)
    dd = d[m].astype(np.float64)
    e1, e2 = c - a, b - a
    P = np.cross(dd, e2)
    det = (e1 * P).sum(1)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / det
        T = oo - a
        u = (T * P).sum(1) * inv
        Q = np.cross(T, e1)
        v = (dd * Q).sum(1) * inv
    w = 1.0 - u - v
    r = np.minimum(np.minimum(u, v), w)
    r[~np.isfinite(r)] = 0.0
    out[m] = r
    return out


def compare_hits(verts, tris, o, d, ids_a, t_a, ids_b, t_b):
    """Returns (mismatch mask, excluded mask).  A mismatch is a compared ray
    whose ids differ or whose t differs by more than 1e-5 relative."""
    near_edge = (edge_distance(verts, tris, ids_a, o, d) < EDGE_EPS) | \
                (edge_distance(verts, tris, ids_b, o, d) < EDGE_EPS)
    tie = (ids_a != ids_b) & (t_a == t_b)
    excluded = near_edge | tie
    same = ids_a == ids_b
    hit = same & (ids_a >= 0)
    tdiff = np.zeros(ids_a.shape[0], bool)
    tdiff[hit] = np.abs(t_a[hit].astype(np.float64) - t_b[hit]) > T_REL * np.abs(t_b[hit].astype(np.float64))
    mismatch = (~same | tdiff) & ~excluded
    return mismatch, excluded


def pixel_agreement(rgb_a, rgb_b):
    diff = np.abs(rgb_a.astype(np.int32) - rgb_b.astype(np.int32)).max(axis=-1)
    return float((diff <= 1).mean()), float((diff == 0).mean()), int(diff.max())


def aa_edge_pixels(oracle, scene, frame, aa_x, aa_y):
    """Output pixels of an anti-aliased frame with at least one sample whose
    primary hit lies within EDGE_EPS of a triangle edge (FP64 barycentrics),
    on the oracle's supersampled camera rays: where a sample may legitimately
    hit a different triangle than the reference's."""
    fine = oracle.supersampled(frame, aa_x, aa_y)
    o, d = oracle.camera_rays(fine["camera"])
    ids, t, _, _ = oracle.OracleScene(scene).closest(o, d)
    near = edge_distance(scene["verts"], scene["tris"], ids, o, d) < EDGE_EPS
    H, W = frame["camera"]["yres"], frame["camera"]["xres"]
    near = near.reshape(H * aa_y, W * aa_x)
    out = np.zeros((H, W), bool)
    for a_x in range(aa_x):
        for a_y in range(aa_y):
            out |= near[a_y::aa_y, a_x::aa_x][:H, :W]
    return out


def glass_cases():
    """(k, keyword arguments of scenes.glass_scene) of the glass-sphere
    frames stored in the golden fixture (keys glass{k}_rgb, glass{k}_args)."""
    import json
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_small.npz"))
    out = []
    k = 0
    while f"glass{k}_args" in g.files:
        out.append((k, json.loads(g[f"glass{k}_args"].tobytes().decode())))
        k += 1
    return out


def tone_cases():
    """(k, tone-map dict, (aa_x, aa_y)) of the tone-mapped golden frames
    (keys {scene}_tone{k}_rgb)."""
    import json
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_small.npz"))
    return [(k, t, tuple(aa)) for k, (t, aa) in enumerate(json.loads(g["tone_cases"].tobytes().decode()))]


def frame_tone_cases():
    """(k, tone-map dict, (aa_x, aa_y)) of the tone maps the reference
    applied to fixed float frames (keys ftone{k}_fimg, ftone{k}_rgb)."""
    import json
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_small.npz"))
    return [(k, t, tuple(aa)) for k, (t, aa) in enumerate(json.loads(g["ftone_cases"].tobytes().decode()))]
