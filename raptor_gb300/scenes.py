"""Seeded synthetic scenes for the five benchmark workloads.

The reference's regression scenes are not available, so these generators
stand in for them.  Every generator is deterministic for a given seed
(numpy PCG64) and uses only IEEE add/mul/div/sqrt in float64 before the
final cast to float32, so the same call yields the same bits on x86 and Arm
(the scale draw of the instanced scene uses exp, the only exception).

A scene is a dict:
  verts  (nv, 3) float32   vertex positions
  tris   (nt, 3) int32     vertex indices (a, b, c); normal = (b-a) x (c-a)
  vattr  (nv, 3) float32   per-vertex colour in [0, 1]
  flags  (nt,)   uint32    bit 0 light, bit 1 transparent
and frames are described by `camera`, `lights` and `material` dicts whose
fields follow the reference's camera / light / coloured_mapper_shader
constructors (raytracer/camera.h:55, raytracer/light.h:17-34,
raytracer/materials/coloured_mapper_shader.h).
"""
from __future__ import annotations

import math

import numpy as np

# Default material: coloured Phong, kd modulated by the per-vertex colour.
DEFAULT_MATERIAL = {"ka": (20.0, 20.0, 20.0), "kd": (204.0, 204.0, 204.0),
                    "ks": (64.0, 64.0, 64.0), "ns": 20.0}


# ----------------------------------------------------------------- meshes

def _icosahedron():
    p = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0],
                  [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
                  [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def geodesic_sphere(freq: int, radius: float = 1.0):
    """Frequency-`freq` geodesic icosphere: 20*freq^2 triangles, 10*freq^2+2
    vertices, outward winding.  Grid points are A*(n-i-j) + B*i + C*j, so a
    point on a shared edge (one weight zero) has the same float64 bits from
    either face and de-duplicates exactly."""
    v, f = _icosahedron()
    n = int(freq)
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    m = (ii + jj) <= n
    ii, jj = ii[m], jj[m]
    kk = n - ii - jj
    # local index of grid point (i, j) within a face
    lid = -np.ones((n + 1, n + 1), dtype=np.int64)
    lid[ii, jj] = np.arange(ii.size)
    # local triangles (up and down)
    tl = []
    for i in range(n):
        for j in range(n - i):
            tl.append((lid[i, j], lid[i + 1, j], lid[i, j + 1]))
            if i + j + 1 < n:
                tl.append((lid[i + 1, j], lid[i + 1, j + 1], lid[i, j + 1]))
    tl = np.array(tl, dtype=np.int64)
    pts, tris = [], []
    for fi, (a, b, c) in enumerate(f):
        A, B, C = v[a], v[b], v[c]
        P = (A[None, :] * kk[:, None] + B[None, :] * ii[:, None]) + C[None, :] * jj[:, None]
        pts.append(P)
        tris.append(tl + fi * ii.size)
    pts = np.concatenate(pts)
    tris = np.concatenate(tris)
    uniq, inv = np.unique(pts, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    nrm = np.sqrt((uniq[:, 0] * uniq[:, 0] + uniq[:, 1] * uniq[:, 1]) + uniq[:, 2] * uniq[:, 2])
    verts = uniq / nrm[:, None] * radius
    tris = inv[tris]
    # orient outward: (b-a) x (c-a) . a > 0
    a, b, c = verts[tris[:, 0]], verts[tris[:, 1]], verts[tris[:, 2]]
    nn = np.cross(b - a, c - a)
    flip = (nn * a).sum(axis=1) < 0
    tris[flip] = tris[flip][:, [0, 2, 1]]
    return verts, tris.astype(np.int32)


def ground_plane(y: float = -1.0, half: float = 20.0):
    verts = np.array([[-half, y, -half], [half, y, -half], [-half, y, half], [half, y, half]], dtype=np.float64)
    tris = np.array([[0, 2, 1], [1, 2, 3]], dtype=np.int32)   # normal +y
    return verts, tris


def diamond_square(size_pow2: int, roughness: float, seed: int) -> np.ndarray:
    """Diamond-square heightfield on a (2^k+1)^2 grid.  Corner heights and
    every displacement are uniform in [-scale, scale]; scale is multiplied
    by `roughness` after each level.  Returns float64 heights (unscaled)."""
    n = int(size_pow2)
    N = n + 1
    rng = np.random.default_rng(seed)
    h = np.zeros((N, N), dtype=np.float64)
    h[0, 0], h[0, n], h[n, 0], h[n, n] = rng.uniform(-1.0, 1.0, 4)
    step, scale = n, 1.0
    while step > 1:
        half = step // 2
        # diamond: square centres
        c = (h[0:n:step, 0:n:step] + h[step::step, 0:n:step]) + (h[0:n:step, step::step] + h[step::step, step::step])
        h[half::step, half::step] = c * 0.25 + rng.uniform(-scale, scale, c.shape)
        # square: edge midpoints, averaging the 3 or 4 neighbours present
        for off in (0, half):
            rows = np.arange(off, N, step) if off == 0 else np.arange(half, N, step)
            cols = np.arange(half, N, step) if off == 0 else np.arange(0, N, step)
            R, Cc = np.meshgrid(rows, cols, indexing="ij")
            acc = np.zeros(R.shape)
            cnt = np.zeros(R.shape)
            for dr, dc in ((-half, 0), (half, 0), (0, -half), (0, half)):
                rr, cc = R + dr, Cc + dc
                ok = (rr >= 0) & (rr < N) & (cc >= 0) & (cc < N)
                acc[ok] += h[rr[ok], cc[ok]]
                cnt[ok] += 1.0
            h[R, Cc] = acc / cnt + rng.uniform(-scale, scale, R.shape)
        step = half
        scale *= roughness
    return h


def heightfield_mesh(h: np.ndarray, extent: float, height: float):
    """Triangulate a heightfield over [0, extent]^2 with heights rescaled to
    [0, height]; two up-facing triangles per cell."""
    N = h.shape[0]
    lo, hi = h.min(), h.max()
    hs = (h - lo) / (hi - lo) * height if hi > lo else np.zeros_like(h)
    sp = extent / (N - 1)
    jj, ii = np.meshgrid(np.arange(N), np.arange(N))
    verts = np.stack([jj * sp, hs, ii * sp], axis=-1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(N - 1), np.arange(N - 1), indexing="ij")
    v00 = (i * N + j).reshape(-1)
    v01 = v00 + 1
    v10 = v00 + N
    v11 = v10 + 1
    t1 = np.stack([v00, v10, v01], axis=1)
    t2 = np.stack([v01, v10, v11], axis=1)
    tris = np.empty((t1.shape[0] * 2, 3), dtype=np.int32)
    tris[0::2] = t1
    tris[1::2] = t2
    return verts, tris, hs


def slope_colours(hs: np.ndarray, spacing: float, height: float) -> np.ndarray:
    """Per-vertex colour from slope and height: grass on flats, rock on
    slopes, snow near the top."""
    gx = np.zeros_like(hs)
    gz = np.zeros_like(hs)
    gx[:, 1:-1] = (hs[:, 2:] - hs[:, :-2]) / (2.0 * spacing)
    gz[1:-1, :] = (hs[2:, :] - hs[:-2, :]) / (2.0 * spacing)
    ny = 1.0 / np.sqrt((gx * gx + gz * gz) + 1.0)
    slope = np.clip((1.0 - ny) * 3.0, 0.0, 1.0)
    grass = np.array([0.25, 0.55, 0.20])
    rock = np.array([0.50, 0.45, 0.40])
    snow = np.array([0.95, 0.95, 0.97])
    col = grass[None, None, :] * (1.0 - slope)[..., None] + rock[None, None, :] * slope[..., None]
    s = np.clip((hs - 0.8 * height) / (0.1 * height), 0.0, 1.0)[..., None]
    col = col * (1.0 - s) + snow[None, None, :] * s
    return col.reshape(-1, 3)


# ---------------------------------------------------------------- cameras

def look_at_camera(eye, target, vfov_deg: float, xres: int, yres: int, background=(0.0, 0.0, 0.0)):
    """Reference camera arguments for a pinhole camera: unit right/up/forward
    axes, image plane at t = 1, half-height tan(vfov/2), half-width scaled by
    the aspect ratio (camera.h:55-62, 121-125)."""
    eye = np.asarray(eye, dtype=np.float64)
    fwd = np.asarray(target, dtype=np.float64) - eye
    fwd = fwd / np.sqrt((fwd[0] * fwd[0] + fwd[1] * fwd[1]) + fwd[2] * fwd[2])
    up = np.array([0.0, 1.0, 0.0])
    right = np.cross(fwd, up)
    right = right / np.sqrt((right[0] * right[0] + right[1] * right[1]) + right[2] * right[2])
    upv = np.cross(right, fwd)
    h = math.tan(math.radians(vfov_deg) / 2.0)
    return {"pos": tuple(float(np.float32(x)) for x in eye),
            "x_axis": tuple(float(np.float32(x)) for x in right),
            "y_axis": tuple(float(np.float32(x)) for x in upv),
            "z_axis": tuple(float(np.float32(x)) for x in fwd),
            "background": tuple(float(x) for x in background),
            "w": float(np.float32(h * xres / yres)), "h": float(np.float32(h)), "t": 1.0,
            "xres": int(xres), "yres": int(yres)}


def point_light(pos, rgb=(255.0, 255.0, 255.0), d=0.0):
    return {"kind": 0, "rgb": tuple(rgb), "pos": tuple(float(x) for x in pos), "dir": (0.0, 0.0, 0.0), "d": float(d)}


def spot_light(pos, direction, s_a, s_b, rgb=(255.0, 255.0, 255.0), d=0.0):
    """Spot light at pos along `direction` (unit), full intensity within
    s_a radians of the axis, none beyond s_b."""
    n = np.asarray(direction, np.float64)
    n = n / np.linalg.norm(n)
    return {"kind": 2, "rgb": tuple(rgb), "pos": tuple(float(x) for x in pos), "dir": tuple(float(x) for x in n),
            "d": d, "s_a": float(s_a), "s_b": float(s_b)}


def directional_light(direction, rgb=(255.0, 255.0, 255.0), d=0.0):
    n = np.asarray(direction, dtype=np.float64)
    n = n / np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])
    return {"kind": 1, "rgb": tuple(rgb), "pos": (0.0, 0.0, 0.0),
            "dir": tuple(float(np.float32(x)) for x in n), "d": float(d)}


def regular_polygon(centre, radius, k, tilt=0.0):
    """k corners of a regular polygon of the given radius around centre, in
    a plane tilted `tilt` radians from horizontal (about x)."""
    a = np.arange(k) * (2.0 * np.pi / k)
    x, z = radius * np.cos(a), radius * np.sin(a)
    y, z = z * np.sin(tilt), z * np.cos(tilt)
    return np.stack([x, y, z], 1) + np.asarray(centre)


def add_area_light(scene, polygon, rgb=(255.0, 255.0, 255.0), d=0.0, spot=None, colour=(1.0, 1.0, 1.0)):
    """The scene with a triangle-defined light appended: the convex polygon
    (k >= 3 corners, in order) fanned into k - 2 triangles flagged as light
    (skipped by shadow rays) with per-vertex attribute `colour`, and the light
    dict (kind 0, or 2 with spot = (direction, s_a, s_b)) whose "tris" lists
    them and whose pos is the corners' mean -- the arguments of the
    reference's triangle-light constructors (light.h:20-21, 27-29)."""
    p = np.asarray(polygon, np.float32)
    k = p.shape[0]
    v0 = scene["verts"].shape[0]
    t0 = scene["tris"].shape[0]
    fan = np.array([[v0, v0 + i, v0 + i + 1] for i in range(1, k - 1)], np.int32)
    flags = scene.get("flags")
    flags = np.zeros(t0, np.uint32) if flags is None else flags
    out = dict(scene)
    out["verts"] = np.ascontiguousarray(np.concatenate([scene["verts"], p]), np.float32)
    out["tris"] = np.ascontiguousarray(np.concatenate([scene["tris"], fan]), np.int32)
    if scene.get("vattr") is not None:
        out["vattr"] = np.ascontiguousarray(
            np.concatenate([scene["vattr"], np.tile(np.asarray(colour, np.float32), (k, 1))]), np.float32)
    out["flags"] = np.concatenate([flags, np.ones(k - 2, np.uint32)])
    if scene.get("mat_of_tri") is not None:
        out["mat_of_tri"] = np.concatenate([scene["mat_of_tri"], np.zeros(k - 2, np.int32)])
    centre = tuple(float(x) for x in p.astype(np.float64).mean(axis=0).astype(np.float32))
    if spot is None:
        light = point_light(centre, rgb, d)
    else:
        light = spot_light(centre, spot[0], spot[1], spot[2], rgb, d)
    light["tris"] = list(range(t0, t0 + k - 2))
    return out, light


def _pack(verts, tris, vattr, flags=None):
    nt = tris.shape[0]
    return {"verts": np.ascontiguousarray(verts, dtype=np.float32),
            "tris": np.ascontiguousarray(tris, dtype=np.int32),
            "vattr": np.ascontiguousarray(vattr, dtype=np.float32),
            "flags": np.zeros(nt, dtype=np.uint32) if flags is None else np.ascontiguousarray(flags, dtype=np.uint32)}


# ------------------------------------------------------------- workloads

def icosphere_scene(freq: int = 32, seed: int = 0, res: int = 512, ground: bool = True):
    """Sphere of 20*freq^2 triangles (r = 1, centred) on a 2-triangle ground at
    y = -1; camera at (0, 0.5, 4) looking at the origin, 60 deg vertical FOV;
    point light at (3, 5, 3); per-vertex colours uniform [0, 1] from `seed`."""
    sv, st = geodesic_sphere(freq)
    if ground:
        gv, gt = ground_plane()
        verts = np.concatenate([sv, gv])
        tris = np.concatenate([st, gt + sv.shape[0]])
    else:
        verts, tris = sv, st
    rng = np.random.default_rng(seed)
    vattr = rng.uniform(0.0, 1.0, (verts.shape[0], 3))
    scene = _pack(verts, tris, vattr)
    frame = {"camera": look_at_camera((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), 60.0, res, res),
             "lights": [point_light((3.0, 5.0, 3.0))], "material": dict(DEFAULT_MATERIAL)}
    return scene, frame


def glass_scene(freq: int = 8, res: int = 64, tran: float = 0.6, ri: float = 1.5, rf_glass: float = 0.2,
                rf_ground: float = 0.3, seed: int = 0):
    """A glass sphere (r = 1 at the origin, material 1: transparency `tran`,
    refractive index `ri`, reflectivity `rf_glass`, a flat kd that ignores
    the vertex colours, triangles flagged transparent so shadow rays pass)
    in front of an opaque sphere (r = 0.6 at (0.4, -0.2, -2.5)), both on a
    40 x 40 ground at y = -1 of reflectivity `rf_ground` (material 0).
    Camera at (0.3, 0.8, 4) looking at (0, -0.2, 0), 50 deg vertical FOV, sky
    background; a point light at (3, 5, 3) and a dimmer directional light.
    The scene dict carries `mat_of_tri`, the frame its `materials` table."""
    v1, t1 = geodesic_sphere(freq)
    v2, t2 = geodesic_sphere(freq)
    v2 = v2 * 0.6 + np.array([0.4, -0.2, -2.5])
    g = np.array([[-20, -1, -20], [20, -1, -20], [20, -1, 20], [-20, -1, 20]], np.float64)
    tg = np.array([[0, 2, 1], [0, 3, 2]])
    verts = np.concatenate([v1, v2, g])
    tris = np.concatenate([t1, t2 + len(v1), tg + len(v1) + len(v2)]).astype(np.int32)
    rng = np.random.default_rng(seed)
    vattr = rng.uniform(0.0, 1.0, (len(verts), 3))
    flags = np.zeros(len(tris), np.uint32)
    flags[:len(t1)] = 2
    mat_of_tri = np.zeros(len(tris), np.int32)
    mat_of_tri[:len(t1)] = 1
    scene = _pack(verts, tris, vattr, flags)
    scene["mat_of_tri"] = mat_of_tri
    base = dict(DEFAULT_MATERIAL)
    mats = [dict(base, rf=rf_ground),
            dict(base, kd=(30.0, 30.0, 40.0), tran=tran, ri=ri, rf=rf_glass, flags=1)]
    cam = look_at_camera((0.3, 0.8, 4.0), (0.0, -0.2, 0.0), 50.0, res, res, background=(110.0, 160.0, 230.0))
    frame = {"camera": cam,
             "lights": [point_light((3.0, 5.0, 3.0)), directional_light((-0.4, -0.8, -0.3), rgb=(80.0, 80.0, 90.0))],
             "materials": mats, "material": mats[0]}
    return scene, frame


def terrain_scene(size_pow2: int = 1024, roughness: float = 0.55, seed: int = 1, xres: int = 1920,
                  yres: int = 1080, extent: float = 1024.0, height: float = 200.0, crop: int = 0):
    """Diamond-square terrain over extent^2 with heights in [0, height]
    (2*size^2 triangles); camera 300 units above the (0, 0) corner looking at
    the centre; directional sun; slope-based per-vertex colour.  crop > 0
    keeps the first crop x crop vertices (same spacing): crop = 725 gives the
    1,048,352-triangle ("1M") variant."""
    h = diamond_square(size_pow2, roughness, seed)
    spacing = extent / size_pow2
    if crop:
        h = h[:crop, :crop]
        extent = spacing * (crop - 1)
    verts, tris, hs = heightfield_mesh(h, extent, height)
    vattr = slope_colours(hs, spacing, height)
    scene = _pack(verts, tris, vattr)
    frame = {"camera": look_at_camera((0.0, 300.0, 0.0), (extent / 2, height / 2, extent / 2), 60.0, xres, yres,
                                      background=(110.0, 160.0, 230.0)),
             "lights": [directional_light((-0.4, -0.8, -0.3))], "material": dict(DEFAULT_MATERIAL)}
    return scene, frame


def _random_quaternions(rng, n):
    """Uniform random rotations by rejection from [-1, 1]^4 (sqrt only)."""
    out = np.empty((n, 4))
    k = 0
    while k < n:
        q = rng.uniform(-1.0, 1.0, (2 * (n - k) + 8, 4))
        r2 = ((q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1]) + q[:, 2] * q[:, 2]) + q[:, 3] * q[:, 3]
        q = q[(r2 > 1e-6) & (r2 <= 1.0)]
        take = min(n - k, q.shape[0])
        out[k:k + take] = q[:take]
        k += take
    r = np.sqrt(((out[:, 0] ** 2 + out[:, 1] ** 2) + out[:, 2] ** 2) + out[:, 3] ** 2)
    return out / r[:, None]


def _quat_to_mat(q):
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)


def instances_scene(n_inst: int = 2000, freq: int = 10, seed: int = 2, xres: int = 1280, yres: int = 720,
                    box: float = 100.0):
    """n_inst randomly placed, rotated and scaled instances of a 20*freq^2
    triangle mesh, half spheres and half cubes (the sphere's vertices pushed
    onto the unit cube), flattened into one mesh.  Positions uniform in
    [0, box]^3, scales log-uniform in [0.5, 5]."""
    sv, st = geodesic_sphere(freq)
    cv = sv / np.abs(sv).max(axis=1, keepdims=True)
    rng = np.random.default_rng(seed)
    kind = rng.integers(0, 2, n_inst)
    pos = rng.uniform(0.0, box, (n_inst, 3))
    scale = np.exp(rng.uniform(math.log(0.5), math.log(5.0), n_inst))
    rot = _quat_to_mat(_random_quaternions(rng, n_inst))
    col = rng.uniform(0.2, 1.0, (n_inst, 3))
    base = np.where(kind[:, None, None] == 0, sv[None], cv[None])            # (n, nv, 3)
    verts = np.einsum("nij,nvj->nvi", rot, base) * scale[:, None, None] + pos[:, None, :]
    nv = sv.shape[0]
    tris = st[None, :, :] + (np.arange(n_inst) * nv)[:, None, None]
    vattr = np.repeat(col[:, None, :], nv, axis=1)
    scene = _pack(verts.reshape(-1, 3), tris.reshape(-1, 3), vattr.reshape(-1, 3))
    frame = {"camera": look_at_camera((box / 2, box / 2, -0.4 * box), (box / 2, box / 2, box / 2), 60.0, xres, yres),
             "lights": [], "material": dict(DEFAULT_MATERIAL), "ao": {"samples": 16, "dist": 5.0, "seed": seed}}
    return scene, frame


def displaced_sphere(freq: int = 50, amp: float = 0.05, seed: int = 4):
    """Geodesic sphere with every vertex moved radially by U[-amp, amp]."""
    v, t = geodesic_sphere(freq)
    rng = np.random.default_rng(seed)
    r = 1.0 + rng.uniform(-amp, amp, v.shape[0])
    v = v * r[:, None]
    col = rng.uniform(0.0, 1.0, v.shape)
    return v, t, col


def adjoint_scene(freq: int = 50, amp: float = 0.05, seed: int = 4, res: int = 256, sigma: float = 0.01):
    """Differentiable-render workload: the displaced sphere, and a target
    mesh perturbed by N(0, sigma^2) per coordinate (same topology/colours)."""
    v, t, col = displaced_sphere(freq, amp, seed)
    rng = np.random.default_rng(seed + 1000)
    vt = v + rng.normal(0.0, sigma, v.shape)
    scene = _pack(v, t, col)
    target = _pack(vt, t, col)
    frame = {"camera": look_at_camera((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), 40.0, res, res),
             "lights": [point_light((3.0, 5.0, 3.0))], "material": dict(DEFAULT_MATERIAL)}
    return scene, target, frame


RESOLUTIONS = [(128, 128), (256, 256), (512, 512), (1024, 768), (1920, 1080)]


def batched_scenes(n: int = 64, seed: int = 3, tri_lo: int = 1000, tri_hi: int = 500000):
    """n independent scenes: icosphere or heightfield, triangle count
    log-uniform in [tri_lo, tri_hi], resolution and ray mix drawn per scene
    (mix 0 = primary + shadow, mix 1 = primary + 4 AO)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        target = math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))
        kind = int(rng.integers(0, 2))
        xres, yres = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        mix = int(rng.integers(0, 2))
        sub_seed = int(rng.integers(0, 2**31 - 1))
        if kind == 0:
            freq = max(1, int(round(math.sqrt(target / 20.0))))
            v, t = geodesic_sphere(freq)
            col = np.random.default_rng(sub_seed).uniform(0.0, 1.0, v.shape)
            scene = _pack(v, t, col)
            cam = look_at_camera((0.0, 0.5, 3.0), (0.0, 0.0, 0.0), 60.0, xres, yres)
            lights = [point_light((3.0, 5.0, 3.0))]
        else:
            m = max(2, int(round(math.sqrt(target / 2.0))))
            p2 = 1 << max(1, (m - 1).bit_length())
            h = diamond_square(p2, 0.55, sub_seed)[: m + 1, : m + 1]
            v, t, hs = heightfield_mesh(h, 100.0, 20.0)
            col = slope_colours(hs, 100.0 / m, 20.0)
            scene = _pack(v, t, col)
            cam = look_at_camera((0.0, 40.0, 0.0), (50.0, 10.0, 50.0), 60.0, xres, yres, background=(110.0, 160.0, 230.0))
            lights = [directional_light((-0.4, -0.8, -0.3))]
        frame = {"camera": cam, "lights": lights if mix == 0 else [], "material": dict(DEFAULT_MATERIAL)}
        if mix == 1:
            frame["ao"] = {"samples": 4, "dist": 2.0, "seed": sub_seed & 0xffff}
        out.append((scene, frame))
    return out
