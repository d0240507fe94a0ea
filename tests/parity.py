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


EPSILON = 1e-3          # the reference's EPSILON: hits at t <= EPSILON are ignored
DET_MIN = 1e-6          # |det| below which triangle::is_intersecting rejects


class OcclusionJudge:
    """FP64 brute-force classification of any-hit rays against every
    triangle of a scene, for explaining occlusion differences ray by ray.

    A triangle blocks a ray when the reference's test accepts it:
    barycentrics inside, t in (EPSILON, tmax), |det| >= 1e-6, and the
    triangle not flagged light or transparent (bvh_node.h:170-190).  In
    FP64 a hit is *robust* when all three barycentrics exceed EDGE_EPS,
    t lies more than 1e-5 relative inside (EPSILON, tmax) and |det| is more
    than 0.1 % away from 1e-6; it is *fragile* when it fails one of those
    margins but not by more than the margin.  classify() returns per ray
    1 (a robust blocker exists: occluded), 0 (no blocker, robust or
    fragile: free) or 2 (only fragile blockers: either answer is
    legitimate in binary32)."""

    def __init__(self, verts, tris, flags=None):
        v = np.asarray(verts, np.float64)
        t = np.asarray(tris, np.int64)
        keep = np.ones(t.shape[0], bool) if flags is None else (np.asarray(flags) & 3) == 0
        t = t[keep]
        a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
        self.a, self.e1, self.e2 = a, c - a, b - a
        self.lo = np.minimum(np.minimum(a, b), c)
        self.hi = np.maximum(np.maximum(a, b), c)

    def _candidates(self, o, d, tmax):
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = 1.0 / d
            t0 = (self.lo - o) * inv
            t1 = (self.hi - o) * inv
        # axis-parallel rays: inside the slab on that axis or not at all
        par = d == 0.0
        if par.any():
            inside = (self.lo[:, par] <= o[par]) & (o[par] <= self.hi[:, par])
            t0[:, par] = np.where(inside, -np.inf, np.inf)
            t1[:, par] = np.where(inside, np.inf, -np.inf)
        tn = np.minimum(t0, t1).max(1)
        tf = np.maximum(t0, t1).min(1)
        slack = 1e-6 * max(1.0, float(tmax))
        return np.nonzero((tn <= tf + slack) & (tf >= -slack) & (tn <= tmax * (1 + 1e-5) + slack))[0]

    def classify(self, ogn, dirs, tmax):
        ogn = np.asarray(ogn, np.float64).reshape(-1, 3)
        dirs = np.asarray(dirs, np.float64).reshape(-1, 3)
        tmax = np.broadcast_to(np.asarray(tmax, np.float64), (ogn.shape[0],))
        out = np.zeros(ogn.shape[0], np.int8)
        for i in range(ogn.shape[0]):
            o, d, tm = ogn[i], dirs[i], float(tmax[i])
            k = self._candidates(o, d, tm)
            if k.size == 0:
                continue
            e1, e2, a = self.e1[k], self.e2[k], self.a[k]
            P = np.cross(d, e2)
            det = (e1 * P).sum(1)
            with np.errstate(divide="ignore", invalid="ignore"):
                T = o - a
                u = (T * P).sum(1) / det
                Q = np.cross(T, e1)
                v = (Q @ d) / det
                t = (e2 * Q).sum(1) / det
            w = 1.0 - u - v
            bary = np.minimum(np.minimum(u, v), w)
            ad = np.abs(det)
            ok = np.isfinite(t) & np.isfinite(bary)
            robust = ok & (bary > EDGE_EPS) & (t > EPSILON * (1 + T_REL)) & (t < tm * (1 - T_REL)) & \
                (ad > DET_MIN * 1.001)
            maybe = ok & (bary > -EDGE_EPS) & (t > EPSILON * (1 - T_REL)) & (t < tm * (1 + T_REL)) & \
                (ad > DET_MIN * 0.999)
            out[i] = 1 if robust.any() else (2 if maybe.any() else 0)
        return out
