"""Python binding of the core's C ABI (include/rtcore.h) through ctypes.

This is plumbing for tests, the smoke check and the benchmark; the product
is the shared library.  Loading fails loudly when the library has not been
built -- there is no CPU fallback.

Bulk arguments may be numpy arrays (host memory) or torch CUDA tensors
(device memory); the library detects which.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

from .build import LIB

RT_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "not built",
          -5: "stack overflow", -6: "iteration limit", -7: "no device", -8: "internal error"}

RT_TRI_LIGHT = 1
RT_TRI_TRANSPARENT = 2
RT_LIGHT_POINT = 0
RT_LIGHT_DIRECTIONAL = 1
RT_MAX_LIGHTS = 8
RT_OPT_COUNT_FETCHES = 1
RT_OPT_RENDER_KERNEL = 2
RT_KERNEL_WAVE = 0
RT_KERNEL_PIXEL = 1
RT_OPT_INTERSECTOR = 3
RT_ISECT_REFERENCE = 0
RT_ISECT_WATERTIGHT = 1
RT_OPT_BUILDER = 4
RT_BUILDER_LBVH = 0
RT_BUILDER_PLOC = 1
RT_BUILDER_HPLOC = 2
RT_OPT_MORTON_BITS = 5


class RtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"rtcore error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class RtRay(C.Structure):
    _fields_ = [("ox", C.c_float), ("oy", C.c_float), ("oz", C.c_float), ("tmax", C.c_float),
                ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float), ("pad", C.c_float)]


class RtHit(C.Structure):
    _fields_ = [("tri", C.c_int32), ("t", C.c_float), ("u", C.c_float), ("v", C.c_float)]


class RtCamera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("x_axis", C.c_float * 3), ("y_axis", C.c_float * 3),
                ("z_axis", C.c_float * 3), ("background", C.c_float * 3), ("w", C.c_float), ("h", C.c_float),
                ("t", C.c_float), ("xres", C.c_int32), ("yres", C.c_int32)]


class RtLight(C.Structure):
    _fields_ = [("kind", C.c_int32), ("rgb", C.c_float * 3), ("pos", C.c_float * 3), ("dir", C.c_float * 3),
                ("d", C.c_float), ("s_a", C.c_float), ("s_b", C.c_float)]


class RtLightShape(C.Structure):
    _fields_ = [("radius", C.c_float), ("ntris", C.c_int32), ("tris", C.POINTER(C.c_int32))]


class RtMaterial(C.Structure):
    _fields_ = [("ka", C.c_float * 3), ("kd", C.c_float * 3), ("ks", C.c_float * 3), ("ns", C.c_float),
                ("rf", C.c_float), ("tran", C.c_float), ("ri", C.c_float), ("flags", C.c_uint32),
                ("rfd", C.c_float), ("td", C.c_float)]


class RtSampling(C.Structure):
    _fields_ = [("soft_samples", C.c_int32), ("diffuse_samples", C.c_int32), ("stream", C.c_int32),
                ("reserved", C.c_int32), ("stream_offset", C.c_int64), ("seed", C.c_uint64)]


RT_STREAM_REFERENCE = 0
RT_STREAM_PIXEL = 1


class RtToneMap(C.Structure):
    _fields_ = [("mode", C.c_int32), ("key", C.c_float), ("xw", C.c_float), ("yw", C.c_float),
                ("desaturate", C.c_int32), ("stretch", C.c_int32), ("gamma", C.c_float)]


class RtMesh(C.Structure):
    _fields_ = [("nverts", C.c_int32), ("ntris", C.c_int32), ("verts", C.POINTER(C.c_float)),
                ("tris", C.POINTER(C.c_int32)), ("tri_rgb", C.POINTER(C.c_uint8)), ("kd", C.c_float * 3),
                ("tri_mat", C.POINTER(C.c_int32)), ("nmat", C.c_int32), ("corner_normals", C.POINTER(C.c_float))]


RT_MESH_AUTO, RT_MESH_OFF, RT_MESH_PLY, RT_MESH_OBJ = 0, 1, 2, 3


class RtRenderStats(C.Structure):
    _fields_ = [("primary_rays", C.c_int64), ("secondary_rays", C.c_int64), ("primary_hits", C.c_int64),
                ("device_ms", C.c_float), ("status", C.c_int32), ("nodes_fetched", C.c_int64),
                ("tris_tested", C.c_int64)]


class RtBvhStats(C.Structure):
    _fields_ = [("nodes", C.c_int64), ("internal_slots", C.c_int64), ("leaf_slots", C.c_int64),
                ("empty_slots", C.c_int64), ("leaf_tris", C.c_int64 * 4)]


RT_JOB_SHADOW = 0
RT_JOB_AO = 1
RT_MAX_JOB_LIGHTS = 2


class RtJob(C.Structure):
    _fields_ = [("scene", C.c_int32), ("mode", C.c_int32), ("camera", RtCamera), ("nlights", C.c_int32),
                ("lights", RtLight * RT_MAX_JOB_LIGHTS), ("material", RtMaterial), ("ao_samples", C.c_int32),
                ("ao_dist", C.c_float), ("ao_seed", C.c_uint32), ("rgb_out", C.c_void_p), ("hit_ids", C.c_void_p)]


class RtTuneConfig(C.Structure):
    _fields_ = [("block_threads", C.c_int32), ("chunk_tiles", C.c_int32), ("tile_w", C.c_int32),
                ("kernel", C.c_int32), ("ms", C.c_float), ("stack_entries", C.c_int32)]


# numpy views of the C structs
RAY_DTYPE = np.dtype([("o", np.float32, 3), ("tmax", np.float32), ("d", np.float32, 3), ("pad", np.float32)])
HIT_DTYPE = np.dtype([("tri", np.int32), ("t", np.float32), ("u", np.float32), ("v", np.float32)])

_lib = None

# (name, restype, argtypes) of every exported entry point, as in rtcore.h
_P = C.c_void_p
SIGNATURES = [
    ("rt_ctx_create", C.c_int32, [C.c_int32, C.POINTER(C.c_void_p)]),
    ("rt_ctx_destroy", C.c_int32, [_P]),
    ("rt_ctx_set_stream", C.c_int32, [_P, _P]),
    ("rt_ctx_synchronize", C.c_int32, [_P]),
    ("rt_ctx_set_option", C.c_int32, [_P, C.c_int32, C.c_int64]),
    ("rt_last_error_string", C.c_char_p, []),
    ("rt_version", C.c_int32, []),
    ("rt_scene_create", C.c_int32, [_P, C.POINTER(C.c_void_p)]),
    ("rt_scene_destroy", C.c_int32, [_P]),
    ("rt_scene_upload", C.c_int32, [_P, _P, C.c_int32, _P, C.c_int32, _P, _P]),
    ("rt_scene_update_vertices", C.c_int32, [_P, _P, C.c_int32]),
    ("rt_bvh_build", C.c_int32, [_P, C.POINTER(C.c_float)]),
    ("rt_bvh_info", C.c_int32, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("rt_bvh_stats_get", C.c_int32, [_P, C.POINTER(RtBvhStats)]),
    ("rt_trace_closest", C.c_int32, [_P, _P, C.c_int32, _P]),
    ("rt_trace_any", C.c_int32, [_P, _P, C.c_int32, _P]),
    ("rt_trace_closest_noalloc", C.c_int32, [_P, _P, C.c_int32, _P]),
    ("rt_scene_refit_vertices", C.c_int32, [_P, _P, C.c_int32, C.POINTER(C.c_float)]),
    ("rt_render", C.c_int32, [_P, C.POINTER(RtCamera), C.POINTER(RtLight), C.c_int32, C.POINTER(RtMaterial), _P, _P,
                              C.POINTER(RtRenderStats)]),
    ("rt_scene_set_materials", C.c_int32, [_P, _P, C.c_int32]),
    ("rt_scene_set_normals", C.c_int32, [_P, _P, C.c_int32]),
    ("rt_sum_sequential_f32", C.c_int32, [_P, _P, C.c_int64, C.POINTER(C.c_float)]),
    ("rt_check_log10", C.c_int32, [_P, C.c_int64, C.c_uint64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("rt_tone_map_image", C.c_int32, [_P, C.POINTER(RtCamera), C.c_int32, C.c_int32, _P, C.POINTER(RtToneMap), _P]),
    ("rt_mesh_load", C.c_int32, [C.c_char_p, C.c_int32, C.POINTER(RtMesh)]),
    ("rt_mesh_parse", C.c_int32, [C.c_char_p, C.c_int64, C.c_int32, C.POINTER(RtMesh)]),
    ("rt_mesh_free", None, [C.POINTER(RtMesh)]),
    ("rt_render_soft_shadows", C.c_int32, [_P, C.POINTER(RtCamera), C.POINTER(RtLight), C.c_int32,
                                           C.POINTER(RtLightShape),
                                           C.POINTER(RtMaterial), C.c_int32, C.c_int32, C.c_int64, _P, _P,
                                           C.POINTER(C.c_int64), C.POINTER(RtRenderStats)]),
    ("rt_render_distributed", C.c_int32, [_P, C.POINTER(RtCamera), C.POINTER(RtLight), C.c_int32,
                                          C.POINTER(RtLightShape), C.POINTER(RtMaterial), C.c_int32,
                                          C.POINTER(RtSampling), _P, _P, C.POINTER(C.c_int64),
                                          C.POINTER(RtRenderStats)]),
    ("rt_render_image", C.c_int32, [_P, C.POINTER(RtCamera), C.POINTER(RtLight), C.c_int32, C.POINTER(RtMaterial),
                                    C.c_int32, _P, C.POINTER(RtRenderStats)]),
    ("rt_render_materials", C.c_int32, [_P, C.POINTER(RtCamera), C.POINTER(RtLight), C.c_int32,
                                        C.POINTER(RtMaterial), C.c_int32, _P, _P, C.POINTER(RtRenderStats)]),
    ("rt_render_tone_mapped", C.c_int32, [_P, C.POINTER(RtCamera), C.c_int32, C.c_int32, C.POINTER(RtLight),
                                          C.c_int32, C.POINTER(RtMaterial), C.c_int32, C.POINTER(RtToneMap), _P,
                                          C.POINTER(RtRenderStats)]),
    ("rt_render_aa", C.c_int32, [_P, C.POINTER(RtCamera), C.c_int32, C.c_int32, C.POINTER(RtLight), C.c_int32,
                                 C.POINTER(RtMaterial), _P, C.POINTER(RtRenderStats)]),
    ("rt_render_ao", C.c_int32, [_P, C.POINTER(RtCamera), C.POINTER(RtMaterial), C.c_int32, C.c_float, C.c_uint32,
                                 _P, _P, _P, C.POINTER(RtRenderStats)]),
    ("rt_scene_update_attributes", C.c_int32, [_P, _P, C.c_int32]),
    ("rt_render_float", C.c_int32, [_P, C.POINTER(RtCamera), C.POINTER(RtLight), C.c_int32, C.POINTER(RtMaterial),
                                    _P, _P, _P, C.POINTER(RtRenderStats)]),
    ("rt_render_adjoint", C.c_int32, [_P, C.POINTER(RtCamera), C.POINTER(RtLight), C.c_int32, C.POINTER(RtMaterial),
                                      _P, _P, _P, C.POINTER(RtRenderStats)]),
    ("rt_batch_create", C.c_int32, [_P, C.POINTER(C.c_void_p)]),
    ("rt_batch_destroy", C.c_int32, [_P]),
    ("rt_batch_add_scene", C.c_int32, [_P, _P, C.c_int32, _P, C.c_int32, _P, _P, C.POINTER(C.c_int32)]),
    ("rt_bvh_build_batched", C.c_int32, [_P, C.POINTER(C.c_float)]),
    ("rt_batch_set_jobs", C.c_int32, [_P, C.POINTER(RtJob), C.c_int32]),
    ("rt_render_batched", C.c_int32, [_P, C.POINTER(RtRenderStats)]),
    ("rt_batch_autotune", C.c_int32, [_P, C.c_int32, C.POINTER(RtTuneConfig)]),
    ("rt_batch_set_config", C.c_int32, [_P, C.POINTER(RtTuneConfig)]),
    ("rt_batch_get_config", C.c_int32, [_P, C.POINTER(RtTuneConfig)]),
]


def lib():
    """Load librtcore.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} is missing: run raptor_gb300.build.build() (there is no CPU fallback)")
        h = C.CDLL(LIB)
        for name, res, args in SIGNATURES:
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        _lib = h
    return _lib


def _check(rc):
    if rc != RT_OK:
        raise RtError(rc, lib().rt_last_error_string().decode())


def ptr(a):
    """Address of a numpy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return C.c_void_p(a.ctypes.data)
    raise TypeError(f"unsupported buffer type {type(a)}")


def make_camera(d) -> RtCamera:
    c = RtCamera()
    for k in ("pos", "x_axis", "y_axis", "z_axis", "background"):
        getattr(c, k)[:] = [float(x) for x in d[k]]
    c.w, c.h, c.t, c.xres, c.yres = d["w"], d["h"], d["t"], d["xres"], d["yres"]
    return c


def make_lights(ls):
    arr = (RtLight * max(1, len(ls)))()
    for i, d in enumerate(ls):
        arr[i].kind = d["kind"]
        arr[i].rgb[:] = list(d["rgb"])
        arr[i].pos[:] = list(d["pos"])
        arr[i].dir[:] = list(d["dir"])
        arr[i].d = d["d"]
        arr[i].s_a = d.get("s_a", 0.0)
        arr[i].s_b = d.get("s_b", 0.0)
    return arr


def make_material(d) -> RtMaterial:
    m = RtMaterial()
    m.ka[:], m.kd[:], m.ks[:] = list(d["ka"]), list(d["kd"]), list(d["ks"])
    m.ns = d["ns"]
    m.rf = d.get("rf", 0.0)
    m.tran = d.get("tran", 0.0)
    m.ri = d.get("ri", 1.0)
    m.flags = d.get("flags", 0)
    m.rfd = d.get("rfd", 0.0)
    m.td = d.get("td", 0.0)
    return m


def make_light_shapes(lights):
    """(RtLightShape array, arrays to keep alive) from light dicts: "r" the
    radius, "tris" the triangles of a triangle-defined light."""
    shapes = (RtLightShape * max(1, len(lights)))()
    keep = []
    for i, l in enumerate(lights):
        shapes[i].radius = float(l.get("r", 0.0))
        if l.get("tris") is not None:
            t = np.ascontiguousarray(l["tris"], np.int32)
            keep.append(t)
            shapes[i].ntris = t.shape[0]
            shapes[i].tris = t.ctypes.data_as(C.POINTER(C.c_int32))
    return shapes, keep


def make_tone_map(d) -> RtToneMap:
    """Tone-map dict -> RtToneMap with camera::tone_map's defaults (key 0.18,
    white point 1/3, 1/3, no desaturation or stretch) and no gamma."""
    t = RtToneMap()
    third = float(np.float32(1.0) / np.float32(3.0))
    t.mode = d.get("mode", 0)
    t.key = d.get("key", 0.18)
    t.xw, t.yw = d.get("xw", third), d.get("yw", third)
    t.desaturate = int(bool(d.get("desaturate", False)))
    t.stretch = int(bool(d.get("stretch", False)))
    t.gamma = d.get("gamma", 0.0)
    return t


def make_materials(ds):
    arr = (RtMaterial * len(ds))()
    for i, d in enumerate(ds):
        arr[i] = make_material(d)
    return arr


def _mesh_dict(m: RtMesh):
    nv, nt = m.nverts, m.ntris
    verts = np.ctypeslib.as_array(m.verts, shape=(max(nv, 1) * 3,))[: nv * 3].reshape(nv, 3).copy()
    tris = np.ctypeslib.as_array(m.tris, shape=(max(nt, 1) * 3,))[: nt * 3].reshape(nt, 3).copy()
    rgb = None
    if m.tri_rgb:
        rgb = np.ctypeslib.as_array(m.tri_rgb, shape=(max(nt, 1) * 3,))[: nt * 3].reshape(nt, 3).copy()
    mat = None
    if m.tri_mat:
        mat = np.ctypeslib.as_array(m.tri_mat, shape=(max(nt, 1),))[:nt].copy()
    cn = None
    if m.corner_normals:
        cn = np.ctypeslib.as_array(m.corner_normals, shape=(max(nt, 1) * 9,))[: nt * 9].reshape(nt, 9).copy()
    return {"verts": verts, "tris": tris, "vattr": None, "flags": None, "tri_rgb": rgb, "kd": tuple(m.kd),
            "tri_mat": mat, "nmat": m.nmat, "corner_normals": cn}


def parse_mesh(data: bytes, fmt: int):
    """rt_mesh_parse on a file's bytes -> scene dict (verts, tris, tri_rgb, kd)."""
    m = RtMesh()
    _check(lib().rt_mesh_parse(data, len(data), fmt, C.byref(m)))
    try:
        return _mesh_dict(m)
    finally:
        lib().rt_mesh_free(C.byref(m))


def load_mesh(path, fmt: int = 0):
    """rt_mesh_load -> scene dict (verts, tris, tri_rgb, kd)."""
    m = RtMesh()
    _check(lib().rt_mesh_load(str(path).encode(), fmt, C.byref(m)))
    try:
        return _mesh_dict(m)
    finally:
        lib().rt_mesh_free(C.byref(m))


def rays_array(ogn, dirs, tmax=None):
    n = ogn.shape[0]
    r = np.zeros(n, RAY_DTYPE)
    r["o"] = ogn
    r["d"] = dirs
    r["tmax"] = np.float32(3.4028234663852886e38) if tmax is None else tmax
    return r


class Context:
    """Owns an rt_context.  Scenes and batches made from it are closed before
    the context itself (the C ABI requires that order)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(lib().rt_ctx_create(device, C.byref(h)))
        self.h = h
        self._children = weakref.WeakSet()

    def set_stream(self, stream_handle):
        """Run on a CUDA stream given by its handle (a non-default stream:
        handle 0 restores the context's own stream)."""
        _check(lib().rt_ctx_set_stream(self.h, C.c_void_p(stream_handle) if stream_handle else None))

    def synchronize(self):
        _check(lib().rt_ctx_synchronize(self.h))

    def set_option(self, option: int, value: int):
        _check(lib().rt_ctx_set_option(self.h, option, value))

    def tone_map_image(self, fimg, camera, tone, aa=(1, 1), rgb=None):
        """rt_tone_map_image: tone map + gamma + downsample of a given float
        frame (rows = y, the aa-supersampled grid of `camera`)."""
        cam = make_camera(camera)
        if rgb is None:
            rgb = np.empty((cam.yres, cam.xres, 3), np.uint8)
        img = np.ascontiguousarray(fimg, np.float32) if isinstance(fimg, np.ndarray) else fimg
        tm = make_tone_map(tone) if tone is not None else None
        _check(lib().rt_tone_map_image(self.h, C.byref(cam), int(aa[0]), int(aa[1]), ptr(img),
                                       C.byref(tm) if tm is not None else None, ptr(rgb)))
        return rgb

    def check_log10(self, n: int, seed: int = 1):
        """(mismatches, undecided) of the tone mapper's float-float log10."""
        bad, und = C.c_int64(), C.c_int64()
        _check(lib().rt_check_log10(self.h, int(n), int(seed), C.byref(bad), C.byref(und)))
        return bad.value, und.value

    def sum_sequential(self, values) -> np.float32:
        """The binary32 sum of values in index order, rounded as a
        sequential loop rounds it (computed on the GPU)."""
        v = np.ascontiguousarray(values, np.float32) if isinstance(values, np.ndarray) else values
        out = C.c_float()
        n = int(v.shape[0]) if hasattr(v, "shape") else len(v)
        _check(lib().rt_sum_sequential_f32(self.h, ptr(v), n, C.byref(out)))
        return np.float32(out.value)

    def close(self):
        if self.h:
            for child in list(self._children):
                child.close()
            lib().rt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    def __init__(self, ctx: Context, scene=None, build: bool = True):
        self.ctx = ctx
        h = C.c_void_p()
        _check(lib().rt_scene_create(ctx.h, C.byref(h)))
        self.h = h
        ctx._children.add(self)
        self.build_ms = None
        if scene is not None:
            self.upload(scene["verts"], scene["tris"], scene.get("vattr"), scene.get("flags"))
            if scene.get("mat_of_tri") is not None:
                self.set_materials(scene["mat_of_tri"])
            if scene.get("corner_normals") is not None:
                self.set_normals(scene["corner_normals"])
            if build:
                self.build()

    def upload(self, verts, tris, vattr=None, flags=None):
        nv = int(verts.shape[0])
        nt = int(tris.shape[0])
        self._keep = (verts, tris, vattr, flags)
        _check(lib().rt_scene_upload(self.h, ptr(verts), nv, ptr(tris), nt, ptr(vattr), ptr(flags)))
        self.nverts, self.ntris = nv, nt

    def set_normals(self, corner_normals):
        """Corner normals per triangle ((n, 3, 3) or n*9 floats), None: none."""
        if corner_normals is None:
            _check(lib().rt_scene_set_normals(self.h, None, 0))
            self._cn = None
            return
        cn = np.ascontiguousarray(corner_normals, np.float32).reshape(-1, 9)
        _check(lib().rt_scene_set_normals(self.h, ptr(cn), int(cn.shape[0])))
        self._cn = cn

    def set_materials(self, mat_of_tri):
        """Material index per triangle (None: every triangle uses material 0)."""
        if mat_of_tri is None:
            _check(lib().rt_scene_set_materials(self.h, None, 0))
            self._mat = None
            return
        mt = np.ascontiguousarray(mat_of_tri, np.int32)
        _check(lib().rt_scene_set_materials(self.h, ptr(mt), int(mt.shape[0])))
        self._mat = mt

    def update_vertices(self, verts):
        _check(lib().rt_scene_update_vertices(self.h, ptr(verts), int(verts.shape[0])))

    def refit_vertices(self, verts) -> float:
        """Move the vertices and refit the existing tree; returns device ms."""
        ms = C.c_float()
        _check(lib().rt_scene_refit_vertices(self.h, ptr(verts), int(verts.shape[0]), C.byref(ms)))
        return ms.value

    def build(self) -> float:
        ms = C.c_float()
        _check(lib().rt_bvh_build(self.h, C.byref(ms)))
        self.build_ms = ms.value
        return ms.value

    def info(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        _check(lib().rt_bvh_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"nodes": a.value, "tri_slots": b.value, "depth": c.value}

    def stats(self):
        st = RtBvhStats()
        _check(lib().rt_bvh_stats_get(self.h, C.byref(st)))
        return {"nodes": st.nodes, "internal_slots": st.internal_slots, "leaf_slots": st.leaf_slots,
                "empty_slots": st.empty_slots, "leaf_tris": list(st.leaf_tris)[1:]}

    def closest(self, rays):
        n = int(rays.shape[0])
        out = np.empty(n, HIT_DTYPE)
        _check(lib().rt_trace_closest(self.h, ptr(rays), n, ptr(out)))
        return out

    def closest_into(self, rays, out):
        _check(lib().rt_trace_closest(self.h, ptr(rays), int(rays.shape[0]), ptr(out)))

    def any(self, rays):
        n = int(rays.shape[0])
        out = np.empty(n, np.uint8)
        _check(lib().rt_trace_any(self.h, ptr(rays), n, ptr(out)))
        return out

    def render(self, frame, rgb=None, ids=None, want_ids=False):
        cam = make_camera(frame["camera"])
        W, H = cam.xres, cam.yres
        if rgb is None:
            rgb = np.empty((H, W, 3), np.uint8)
        if ids is None and want_ids:
            ids = np.empty((H, W), np.int32)
        st = RtRenderStats()
        mat = make_material(frame["material"] if "material" in frame else frame["materials"][0])
        ao = frame.get("ao")
        if ao:
            cnt = np.empty((H, W), np.int32) if want_ids else None
            _check(lib().rt_render_ao(self.h, C.byref(cam), C.byref(mat), ao["samples"], ao["dist"], ao["seed"],
                                      ptr(rgb), ptr(ids), ptr(cnt), C.byref(st)))
            return {"rgb": rgb, "ids": ids, "ao_count": cnt, "stats": st}
        ls = make_lights(frame["lights"])
        if frame.get("materials"):
            table = make_materials(frame["materials"])
            _check(lib().rt_render_materials(self.h, C.byref(cam), ls, len(frame["lights"]), table, len(table),
                                             ptr(rgb), ptr(ids), C.byref(st)))
        else:
            _check(lib().rt_render(self.h, C.byref(cam), ls, len(frame["lights"]), C.byref(mat), ptr(rgb), ptr(ids),
                                   C.byref(st)))
        return {"rgb": rgb, "ids": ids, "stats": st}

    def render_tone_mapped(self, frame, tone=None, aa=(1, 1), rgb=None):
        """Frame on the aa grid, tone mapped and gamma corrected (tone dict or
        None), averaged to RGB8; frame["materials"] or frame["material"]."""
        cam = make_camera(frame["camera"])
        if rgb is None:
            rgb = np.empty((cam.yres, cam.xres, 3), np.uint8)
        st = RtRenderStats()
        ls = make_lights(frame["lights"])
        table = make_materials(frame["materials"] if frame.get("materials") else [frame["material"]])
        tm = make_tone_map(tone) if tone is not None else None
        _check(lib().rt_render_tone_mapped(self.h, C.byref(cam), int(aa[0]), int(aa[1]), ls, len(frame["lights"]),
                                           table, len(table), C.byref(tm) if tm is not None else None, ptr(rgb),
                                           C.byref(st)))
        return {"rgb": rgb, "stats": st}

    def render_image(self, frame, aa=(1, 1), fimg=None):
        """rt_render_image: the camera's float image on the aa-supersampled
        grid (rows = y), frame["materials"] or frame["material"]; fimg: host
        array or device tensor, allocated on the host when None."""
        cam = make_camera(frame["camera"])
        cam.xres, cam.yres = cam.xres * int(aa[0]), cam.yres * int(aa[1])
        if fimg is None:
            fimg = np.empty((cam.yres, cam.xres, 3), np.float32)
        st = RtRenderStats()
        ls = make_lights(frame["lights"])
        table = make_materials(frame["materials"] if frame.get("materials") else [frame["material"]])
        _check(lib().rt_render_image(self.h, C.byref(cam), ls, len(frame["lights"]), table, len(table), ptr(fimg),
                                     C.byref(st)))
        return {"fimg": fimg, "stats": st}

    def render_soft(self, frame, samples, stream_offset=0, rgb=None, fimg=None, want_float=False):
        """rt_render_soft_shadows: `samples` soft-shadow rays per spherical
        light (radius: each light dict's "r", default 0) or triangle-defined
        light (a light dict's "tris": indices of the scene's triangles),
        drawing the reference's random stream from stream_offset.  rgb /
        fimg: host arrays or device tensors (allocated on the host when
        None; fimg only with want_float).  Returns rgb, fimg, stats and
        stream_end."""
        cam = make_camera(frame["camera"])
        if rgb is None:
            rgb = np.empty((cam.yres, cam.xres, 3), np.uint8)
        if fimg is None and want_float:
            fimg = np.empty((cam.yres, cam.xres, 3), np.float32)
        ls = make_lights(frame["lights"])
        shapes, keep = make_light_shapes(frame["lights"])
        table = make_materials(frame["materials"] if frame.get("materials") else [frame["material"]])
        st = RtRenderStats()
        end = C.c_int64(0)
        _check(lib().rt_render_soft_shadows(self.h, C.byref(cam), ls, len(frame["lights"]), shapes, table,
                                            len(table), int(samples), int(stream_offset), ptr(rgb), ptr(fimg),
                                            C.byref(end), C.byref(st)))
        return {"rgb": rgb, "fimg": fimg, "stats": st, "stream_end": end.value}

    def render_distributed(self, frame, soft=1, diffuse=0, stream=RT_STREAM_REFERENCE, offset=0, seed=0, rgb=None,
                           fimg=None, want_float=False):
        """rt_render_distributed: the reference's ray tree with SOFT_SHADOW =
        soft and DIFFUSE_REFLECTIONS = diffuse (materials' "rfd" / "td"),
        numbers from the reference's stream at `offset` or from per-pixel
        streams keyed by `seed`.  Returns rgb, fimg, stats and stream_end
        (the generator's position after the frame, or the numbers drawn)."""
        cam = make_camera(frame["camera"])
        if rgb is None:
            rgb = np.empty((cam.yres, cam.xres, 3), np.uint8)
        if fimg is None and want_float:
            fimg = np.empty((cam.yres, cam.xres, 3), np.float32)
        ls = make_lights(frame["lights"])
        shapes, keep = make_light_shapes(frame["lights"])
        table = make_materials(frame["materials"] if frame.get("materials") else [frame["material"]])
        smp = RtSampling(int(soft), int(diffuse), int(stream), 0, int(offset), int(seed))
        st = RtRenderStats()
        end = C.c_int64(0)
        _check(lib().rt_render_distributed(self.h, C.byref(cam), ls, len(frame["lights"]), shapes, table, len(table),
                                           C.byref(smp), ptr(rgb), ptr(fimg), C.byref(end), C.byref(st)))
        return {"rgb": rgb, "fimg": fimg, "stats": st, "stream_end": end.value}

    def render_aa(self, frame, aa_x, aa_y, rgb=None):
        """Anti-aliased frame: aa_x * aa_y rays per output pixel, averaged."""
        cam = make_camera(frame["camera"])
        if rgb is None:
            rgb = np.empty((cam.yres, cam.xres, 3), np.uint8)
        st = RtRenderStats()
        ls = make_lights(frame["lights"])
        _check(lib().rt_render_aa(self.h, C.byref(cam), int(aa_x), int(aa_y), ls, len(frame["lights"]),
                                  C.byref(make_material(frame["material"])), ptr(rgb), C.byref(st)))
        return {"rgb": rgb, "stats": st}

    def update_attributes(self, vattr):
        _check(lib().rt_scene_update_attributes(self.h, ptr(vattr), int(vattr.shape[0])))

    def render_float(self, frame, fimg, ids=None, occl=None):
        """Unclipped float frame into device buffers (torch tensors)."""
        cam = make_camera(frame["camera"])
        ls = make_lights(frame["lights"])
        st = RtRenderStats()
        _check(lib().rt_render_float(self.h, C.byref(cam), ls, len(frame["lights"]),
                                     C.byref(make_material(frame["material"])), ptr(fimg), ptr(ids), ptr(occl),
                                     C.byref(st)))
        return st

    def render_adjoint(self, frame, dldpix, gpos, gcol):
        cam = make_camera(frame["camera"])
        ls = make_lights(frame["lights"])
        st = RtRenderStats()
        _check(lib().rt_render_adjoint(self.h, C.byref(cam), ls, len(frame["lights"]),
                                       C.byref(make_material(frame["material"])), ptr(dldpix), ptr(gpos), ptr(gcol),
                                       C.byref(st)))
        return st

    def close(self):
        if self.h and self.ctx.h:
            lib().rt_scene_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_job(scene_index, frame, rgb_dev, ids_dev=None) -> RtJob:
    """Job for one frame dict (scenes.* format) rendering into device buffers."""
    j = RtJob()
    j.scene = scene_index
    j.camera = make_camera(frame["camera"])
    j.material = make_material(frame["material"])
    ao = frame.get("ao")
    if ao:
        j.mode = RT_JOB_AO
        j.ao_samples, j.ao_dist, j.ao_seed = ao["samples"], ao["dist"], ao["seed"]
        j.nlights = 0
    else:
        j.mode = RT_JOB_SHADOW
        ls = frame["lights"]
        if len(ls) > RT_MAX_JOB_LIGHTS:
            raise ValueError("too many lights for a batch job")
        j.nlights = len(ls)
        arr = make_lights(ls)
        for i in range(len(ls)):
            j.lights[i] = arr[i]
    j.rgb_out = ptr(rgb_dev).value
    j.hit_ids = ptr(ids_dev).value if ids_dev is not None else None
    return j


class Batch:
    """Many scenes in one persistent, graph-captured launch."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        _check(lib().rt_batch_create(ctx.h, C.byref(h)))
        self.h = h
        ctx._children.add(self)
        self._keep = []
        self.build_ms = None

    def add_scene(self, scene) -> int:
        idx = C.c_int32()
        v, t = scene["verts"], scene["tris"]
        a, f = scene.get("vattr"), scene.get("flags")
        self._keep.append((v, t, a, f))
        _check(lib().rt_batch_add_scene(self.h, ptr(v), int(v.shape[0]), ptr(t), int(t.shape[0]), ptr(a), ptr(f),
                                        C.byref(idx)))
        return idx.value

    def build(self) -> float:
        ms = C.c_float()
        _check(lib().rt_bvh_build_batched(self.h, C.byref(ms)))
        self.build_ms = ms.value
        return ms.value

    def set_jobs(self, jobs):
        arr = (RtJob * max(1, len(jobs)))(*jobs)
        self._jobs = arr
        _check(lib().rt_batch_set_jobs(self.h, arr, len(jobs)))

    def render(self, stats=True):
        st = RtRenderStats()
        _check(lib().rt_render_batched(self.h, C.byref(st) if stats else None))
        return st

    def autotune(self, reps=3):
        cfg = RtTuneConfig()
        _check(lib().rt_batch_autotune(self.h, reps, C.byref(cfg)))
        return {"block_threads": cfg.block_threads, "chunk_tiles": cfg.chunk_tiles, "tile_w": cfg.tile_w,
                "kernel": "wave" if cfg.kernel == RT_KERNEL_WAVE else "pixel", "ms": cfg.ms,
                "stack_entries": cfg.stack_entries}

    def set_config(self, block_threads=128, chunk_tiles=1, tile_w=8, kernel=0, stack_entries=48):
        cfg = RtTuneConfig(block_threads, chunk_tiles, tile_w, kernel, 0.0, stack_entries)
        _check(lib().rt_batch_set_config(self.h, C.byref(cfg)))

    def close(self):
        if self.h and self.ctx.h:
            lib().rt_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
