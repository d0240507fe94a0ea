"""ctypes front end of the oracle libraries -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_build/librtoracle.so (the C restatement of the reference's
hot path) and, where it was built, oracle/_ref/libraptor_ref.so (the
reference's own sources behind a harness).  Only tests, the smoke check and
the CPU-baseline leg of the benchmark import this module; the product never
does.  `build()` compiles both.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "librtoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libraptor_ref.so")
# the reference built with soft shadows on (SOFT_SHADOW = REF_SOFT_SAMPLES)
REF_SOFT_SAMPLES = 16
REF_SOFT_SO = os.path.join(HERE, "_ref", f"libraptor_ref_soft{REF_SOFT_SAMPLES}.so")
# ... and with diffuse reflections too (DIFFUSE_REFLECTIONS = REF_DIFFUSE_SAMPLES)
REF_DIFFUSE_SAMPLES = 16
REF_DIFFUSE_SO = os.path.join(HERE, "_ref",
                              f"libraptor_ref_soft{REF_SOFT_SAMPLES}_diffuse{REF_DIFFUSE_SAMPLES}.so")
# RAPTor source tree (the directory holding common/ and raytracer/); the
# RAPTOR_REF environment variable overrides the default checkout location.
REF_SRC = os.environ.get("RAPTOR_REF", "/root/reference/RAPTor")


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("x_axis", C.c_float * 3), ("y_axis", C.c_float * 3),
                ("z_axis", C.c_float * 3), ("background", C.c_float * 3), ("w", C.c_float),
                ("h", C.c_float), ("t", C.c_float), ("xres", C.c_int32), ("yres", C.c_int32)]


class Light(C.Structure):
    _fields_ = [("kind", C.c_int32), ("rgb", C.c_float * 3), ("pos", C.c_float * 3), ("dir", C.c_float * 3),
                ("d", C.c_float), ("s_a", C.c_float), ("s_b", C.c_float), ("r", C.c_float),
                ("ntris", C.c_int32), ("tris", C.POINTER(C.c_int32))]


class Material(C.Structure):
    _fields_ = [("ka", C.c_float * 3), ("kd", C.c_float * 3), ("ks", C.c_float * 3), ("ns", C.c_float),
                ("rf", C.c_float), ("tran", C.c_float), ("ri", C.c_float), ("flags", C.c_uint32),
                ("rfd", C.c_float), ("td", C.c_float)]


class Sampling(C.Structure):
    _fields_ = [("soft", C.c_int32), ("diffuse", C.c_int32), ("stream", C.c_int32), ("reserved", C.c_int32),
                ("offset", C.c_int64), ("seed", C.c_uint64)]


STREAM_REFERENCE = 0
STREAM_PIXEL = 1


class ToneMap(C.Structure):
    _fields_ = [("mode", C.c_int32), ("key", C.c_float), ("xw", C.c_float), ("yw", C.c_float),
                ("desaturate", C.c_int32), ("stretch", C.c_int32), ("gamma", C.c_float),
                ("cam_w", C.c_float), ("cam_h", C.c_float), ("cam_t", C.c_float)]


def make_tone_map(d, camera=None):
    """Tone-map dict -> ToneMap; the defaults are camera::tone_map's
    (key 0.18, white point 1/3, 1/3, no desaturation or stretch) and no
    gamma correction."""
    t = ToneMap()
    t.mode = d.get("mode", 0)
    t.key = d.get("key", 0.18)
    t.xw = d.get("xw", float(np.float32(1.0) / np.float32(3.0)))
    t.yw = d.get("yw", float(np.float32(1.0) / np.float32(3.0)))
    t.desaturate = int(bool(d.get("desaturate", False)))
    t.stretch = int(bool(d.get("stretch", False)))
    t.gamma = d.get("gamma", 0.0)
    if camera is not None:
        t.cam_w, t.cam_h, t.cam_t = camera["w"], camera["h"], camera["t"]
    return t


def make_camera(d):
    c = Camera()
    for k in ("pos", "x_axis", "y_axis", "z_axis", "background"):
        getattr(c, k)[:] = [float(x) for x in d[k]]
    c.w, c.h, c.t, c.xres, c.yres = d["w"], d["h"], d["t"], d["xres"], d["yres"]
    return c


def make_lights(ls):
    """Light array from light dicts; "tris" (triangle indices) makes a
    triangle-defined light, its index arrays kept alive on the array."""
    arr = (Light * max(1, len(ls)))()
    arr._tris = []
    for i, d in enumerate(ls):
        arr[i].kind = d["kind"]
        arr[i].rgb[:] = list(d["rgb"])
        arr[i].pos[:] = list(d["pos"])
        arr[i].dir[:] = list(d["dir"])
        arr[i].d = d["d"]
        arr[i].s_a = d.get("s_a", 0.0)
        arr[i].s_b = d.get("s_b", 0.0)
        arr[i].r = d.get("r", 0.0)
        if d.get("tris") is not None:
            t = np.ascontiguousarray(d["tris"], np.int32)
            arr._tris.append(t)
            arr[i].ntris = t.shape[0]
            arr[i].tris = t.ctypes.data_as(C.POINTER(C.c_int32))
    return arr


def make_material(d):
    m = Material()
    m.ka[:], m.kd[:], m.ks[:] = list(d["ka"]), list(d["kd"]), list(d["ks"])
    m.ns = d["ns"]
    m.rf = d.get("rf", 0.0)
    m.tran = d.get("tran", 0.0)
    m.ri = d.get("ri", 1.0)
    m.flags = d.get("flags", 0)
    m.rfd = d.get("rfd", 0.0)
    m.td = d.get("td", 0.0)
    return m


def make_materials(ds):
    arr = (Material * len(ds))()
    for i, d in enumerate(ds):
        arr[i] = make_material(d)
    return arr


def build(verbose: bool = False) -> None:
    """Compile the C restatement; compile the reference harness too when the
    reference tree is present and the host is x86-64."""
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-o", ORACLE_SO,
           os.path.join(HERE, "rtoracle.c"), "-lm", "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    if os.path.isdir(REF_SRC) and platform.machine() in ("x86_64", "AMD64"):
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "refbuild"), f"REF={REF_SRC}", "-j8"], check=True,
                       capture_output=not verbose)
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "refbuild"), f"REF={REF_SRC}",
                        f"SOFT={REF_SOFT_SAMPLES}", "-j8"], check=True, capture_output=not verbose)
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "refbuild"), f"REF={REF_SRC}",
                        f"SOFT={REF_SOFT_SAMPLES}", f"DIFFUSE={REF_DIFFUSE_SAMPLES}", "-j8"], check=True,
                       capture_output=not verbose)


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)
_U32 = C.POINTER(C.c_uint32)
_U8 = C.POINTER(C.c_uint8)


def _declare(lib, prefix):
    lib[prefix + "scene_build"].restype = C.c_double
    lib[prefix + "scene_build"].argtypes = [C.c_void_p]
    lib[prefix + "scene_destroy"].argtypes = [C.c_void_p]
    lib[prefix + "trace_closest"].argtypes = [C.c_void_p, _F, _F, C.c_int32, _I, _F, _F, _F]
    lib[prefix + "trace_any"].argtypes = [C.c_void_p, _F, _F, _F, C.c_int32, _U8]
    lib[prefix + "camera_rays"].argtypes = [C.POINTER(Camera), C.c_int32, C.c_int32, C.c_int32, C.c_int32, _F, _F]
    lib[prefix + "morton_code"].restype = C.c_int32
    lib[prefix + "morton_code"].argtypes = [C.c_float] * 6


class _Lib:
    def __init__(self, path):
        self.h = C.CDLL(path)

    def __getitem__(self, k):
        return getattr(self.h, k)


class _SceneBase:
    prefix = ""

    def closest(self, ogn, dir):
        ogn = np.ascontiguousarray(ogn, dtype=np.float32).reshape(-1, 3)
        dir = np.ascontiguousarray(dir, dtype=np.float32).reshape(-1, 3)
        n = ogn.shape[0]
        ids = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float32) for _ in range(3))
        rc = self.lib[self.prefix + "trace_closest"](self.h, _p(ogn, C.c_float), _p(dir, C.c_float), n,
                                                     _p(ids, C.c_int32), _p(t, C.c_float), _p(u, C.c_float),
                                                     _p(v, C.c_float))
        if rc != 0:
            raise RuntimeError("trace_closest failed")
        return ids, t, u, v

    def any(self, ogn, dir, tmax):
        ogn = np.ascontiguousarray(ogn, dtype=np.float32).reshape(-1, 3)
        dir = np.ascontiguousarray(dir, dtype=np.float32).reshape(-1, 3)
        tmax = np.ascontiguousarray(np.broadcast_to(np.asarray(tmax, np.float32), (ogn.shape[0],)))
        occ = np.empty(ogn.shape[0], np.uint8)
        rc = self.lib[self.prefix + "trace_any"](self.h, _p(ogn, C.c_float), _p(dir, C.c_float), _p(tmax, C.c_float),
                                                 ogn.shape[0], _p(occ, C.c_uint8))
        if rc != 0:
            raise RuntimeError("trace_any failed")
        return occ

    def close(self):
        if self.h:
            self.lib[self.prefix + "scene_destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_oracle = None
_ref = None


def oracle_lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            build()
        lib = _Lib(ORACLE_SO)
        _declare(lib, "ro_")
        lib["ro_scene_create"].restype = C.c_void_p
        lib["ro_scene_create"].argtypes = [_F, C.c_int32, _I, C.c_int32, _F, _U32]
        lib["ro_scene_node_count"].restype = C.c_int32
        lib["ro_scene_node_count"].argtypes = [C.c_void_p]
        lib["ro_render"].restype = C.c_int64
        lib["ro_render"].argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(Light), C.c_int32, C.POINTER(Material),
                                     C.c_int32, C.c_int32, C.c_int32, _U8, _I, _U8, _F]
        lib["ro_render_mt"].restype = C.c_int64
        lib["ro_render_mt"].argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(Light), C.c_int32,
                                        C.POINTER(Material), C.c_int32, C.c_int32, C.c_int32, C.c_int32, _U8, _I,
                                        _U8, _F]
        lib["ro_scene_set_normals"].restype = C.c_int32
        lib["ro_scene_set_normals"].argtypes = [C.c_void_p, _F]
        lib["ro_scene_set_materials"].restype = C.c_int32
        lib["ro_scene_set_materials"].argtypes = [C.c_void_p, _I]
        lib["ro_tone_map_frame"].restype = C.c_int32
        lib["ro_tone_map_frame"].argtypes = [_F, C.c_int32, C.c_int32, C.POINTER(ToneMap)]
        lib["ro_render_ao"].restype = C.c_int64
        lib["ro_render_ao"].argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(Material), C.c_int32, C.c_float,
                                        C.c_uint32, C.c_int32, C.c_int32, C.c_int32, _U8, _I, _I]
        lib["ro_ao_rays"].argtypes = [_F, _F, C.c_uint32, C.c_int32, C.c_uint32, _F, _F]
        lib["ro_philox4x32"].argtypes = [_U32, C.c_uint32, C.c_uint32, _U32]
        lib["ro_render_soft"].restype = C.c_int64
        lib["ro_render_soft"].argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(Light), C.c_int32,
                                          C.POINTER(Material), C.c_int32, C.c_int32, C.c_int64, C.c_int32, _U8, _I,
                                          _F, C.POINTER(C.c_int64)]
        lib["ro_ref_random"].restype = None
        lib["ro_ref_random"].argtypes = [C.c_int64, C.c_int32, _F]
        lib["ro_render_distributed"].restype = C.c_int64
        lib["ro_render_distributed"].argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(Light), C.c_int32,
                                                 C.POINTER(Material), C.c_int32, C.POINTER(Sampling), C.c_int32,
                                                 _U8, _I, _F, C.POINTER(C.c_int64)]
        lib["ro_pixel_stream"].restype = C.c_float
        lib["ro_pixel_stream"].argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint32]
        lib["ro_tree_child"].restype = C.c_uint64
        lib["ro_tree_child"].argtypes = [C.c_uint64, C.c_int32, C.c_int32]
        lib["ro_area_light_rays"].restype = C.c_int32
        lib["ro_area_light_rays"].argtypes = [C.c_int32, C.c_int32, _I]
        lib["ro_lut_cos"].restype = C.c_float
        lib["ro_lut_cos"].argtypes = [C.c_float]
        lib["ro_lut_sin"].restype = C.c_float
        lib["ro_lut_sin"].argtypes = [C.c_float]
        lib["ro_pixel_secondary_rays"].restype = C.c_int32
        lib["ro_pixel_secondary_rays"].argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(Light), C.c_int32,
                                                   C.c_int32, C.c_float, C.c_uint32, C.c_int32, C.c_int32, _I, _F,
                                                   _F, _F]
        _oracle = lib
    return _oracle


def ref_available() -> bool:
    return os.path.exists(REF_SO)


_ref_variants = {}


def _ref_variant(path):
    if path not in _ref_variants:
        lib = _load_ref(path)
        lib["rref_random"].restype = None
        lib["rref_random"].argtypes = [C.c_int32, _F]
        lib["rref_lut_cos"].restype = C.c_float
        lib["rref_lut_cos"].argtypes = [C.c_float]
        lib["rref_lut_sin"].restype = C.c_float
        lib["rref_lut_sin"].argtypes = [C.c_float]
        lib["rref_soft_shadow_samples"].restype = C.c_int32
        lib["rref_diffuse_samples"].restype = C.c_int32
        _ref_variants[path] = lib
    return _ref_variants[path]


def ref_soft_lib():
    """The reference built with SOFT_SHADOW = REF_SOFT_SAMPLES (x86 only).
    Its random generator is process-wide: every soft frame it renders moves
    it on."""
    return _ref_variant(REF_SOFT_SO)


def ref_diffuse_lib():
    """The reference built with SOFT_SHADOW = REF_SOFT_SAMPLES and
    DIFFUSE_REFLECTIONS = REF_DIFFUSE_SAMPLES (x86 only); its own generator,
    separate from ref_soft_lib's."""
    return _ref_variant(REF_DIFFUSE_SO)


def ref_lib():
    global _ref
    if _ref is None:
        _ref = _load_ref(REF_SO)
    return _ref


def _load_ref(path):
    if True:
        lib = _Lib(path)
        _declare(lib, "rref_")
        lib["rref_scene_create"].restype = C.c_void_p
        lib["rref_scene_create"].argtypes = [_F, C.c_int32, _I, C.c_int32, _F, _U32, C.POINTER(Material)]
        lib["rref_scene_create_mt"].restype = C.c_void_p
        lib["rref_scene_create_mt"].argtypes = [_F, C.c_int32, _I, C.c_int32, _F, _U32, C.POINTER(Material),
                                                C.c_int32, _I]
        lib["rref_render"].restype = C.c_double
        lib["rref_render"].argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(Light), C.c_int32, _U8]
        lib["rref_render_aa"].restype = C.c_double
        lib["rref_render_aa"].argtypes = [C.c_void_p, C.POINTER(Camera), C.c_int32, C.c_int32, C.POINTER(Light),
                                          C.c_int32, _U8]
        lib["rref_parse_mesh"].restype = C.c_int64
        lib["rref_parse_mesh"].argtypes = [C.c_char_p, C.c_int32, _F, C.c_int64, C.POINTER(C.c_int32)]
        lib["rref_parse_and_render"].restype = C.c_int64
        lib["rref_parse_and_render"].argtypes = [C.c_char_p, C.c_int32, C.POINTER(Camera), C.POINTER(Light),
                                                 C.c_int32, _U8]
        lib["rref_tone_map_image"].restype = None
        lib["rref_tone_map_image"].argtypes = [C.POINTER(Camera), C.c_int32, C.c_int32, _F, C.POINTER(ToneMap), _U8]
        lib["rref_render_tone_mapped"].restype = C.c_double
        lib["rref_render_tone_mapped"].argtypes = [C.c_void_p, C.POINTER(Camera), C.c_int32, C.c_int32,
                                                   C.POINTER(Light), C.c_int32, C.POINTER(ToneMap), _U8]
    return lib


def _scene_arrays(scene):
    v = np.ascontiguousarray(scene["verts"], np.float32)
    t = np.ascontiguousarray(scene["tris"], np.int32)
    a = scene.get("vattr")
    a = None if a is None else np.ascontiguousarray(a, np.float32)
    f = scene.get("flags")
    f = None if f is None else np.ascontiguousarray(f, np.uint32)
    return v, t, a, f


class OracleScene(_SceneBase):
    """The C restatement, built on construction."""
    prefix = "ro_"

    def __init__(self, scene):
        self.lib = oracle_lib()
        v, t, a, f = _scene_arrays(scene)
        self._keep = (v, t, a, f)
        self.h = self.lib["ro_scene_create"](_p(v, C.c_float), v.shape[0], _p(t, C.c_int32), t.shape[0],
                                             _p(a, C.c_float), _p(f, C.c_uint32))
        if not self.h:
            raise ValueError("invalid scene")
        if scene.get("mat_of_tri") is not None:
            mt = np.ascontiguousarray(scene["mat_of_tri"], np.int32)
            self._keep = self._keep + (mt,)
            if self.lib["ro_scene_set_materials"](self.h, _p(mt, C.c_int32)) != 0:
                raise MemoryError("oracle materials failed")
        if scene.get("corner_normals") is not None:
            cn = np.ascontiguousarray(scene["corner_normals"], np.float32)
            self._keep = self._keep + (cn,)
            if self.lib["ro_scene_set_normals"](self.h, _p(cn, C.c_float)) != 0:
                raise MemoryError("oracle normals failed")
        self.build_seconds = self.lib["ro_scene_build"](self.h)
        if self.build_seconds < 0:
            raise MemoryError("oracle build failed")

    def node_count(self):
        return self.lib["ro_scene_node_count"](self.h)

    def render_soft(self, frame, samples, stream_offset=0, threads=1, want_ids=False, want_float=False):
        """ro_render_soft: the whole frame with `samples` soft-shadow rays per
        spherical light, drawing the reference's random stream from position
        stream_offset.  frame["materials"] or frame["material"]."""
        cam = make_camera(frame["camera"])
        W, H = cam.xres, cam.yres
        rgb = np.zeros((H, W, 3), np.uint8)
        ids = np.full((H, W), -2, np.int32) if want_ids else None
        fimg = np.zeros((H, W, 3), np.float32) if want_float else None
        ls = make_lights(frame["lights"])
        table = make_materials(frame["materials"] if frame.get("materials") else [frame["material"]])
        end = C.c_int64(0)
        n = self.lib["ro_render_soft"](self.h, C.byref(cam), ls, len(frame["lights"]), table, len(table), int(samples),
                                       int(stream_offset), threads, _p(rgb, C.c_uint8), _p(ids, C.c_int32),
                                       _p(fimg, C.c_float), C.byref(end))
        if n < 0:
            raise ValueError("oracle soft-shadow render refused its arguments")
        return {"rgb": rgb, "ids": ids, "fimg": fimg, "rays": n, "stream_end": end.value}

    def render_distributed(self, frame, soft=1, diffuse=0, stream=STREAM_REFERENCE, offset=0, seed=0, threads=1,
                           want_ids=False, want_float=False):
        """ro_render_distributed: the reference's ray tree with SOFT_SHADOW =
        soft and DIFFUSE_REFLECTIONS = diffuse, numbers from the reference's
        generator at position `offset` (serial) or from per-pixel streams
        keyed by `seed`.  Returns rgb, ids, fimg, rays and drawn (numbers
        the frame drew)."""
        cam = make_camera(frame["camera"])
        W, H = cam.xres, cam.yres
        rgb = np.zeros((H, W, 3), np.uint8)
        ids = np.full((H, W), -2, np.int32) if want_ids else None
        fimg = np.zeros((H, W, 3), np.float32) if want_float else None
        ls = make_lights(frame["lights"])
        table = make_materials(frame["materials"] if frame.get("materials") else [frame["material"]])
        smp = Sampling(int(soft), int(diffuse), int(stream), 0, int(offset), int(seed))
        drawn = C.c_int64(0)
        n = self.lib["ro_render_distributed"](self.h, C.byref(cam), ls, len(frame["lights"]), table, len(table),
                                              C.byref(smp), int(threads), _p(rgb, C.c_uint8), _p(ids, C.c_int32),
                                              _p(fimg, C.c_float), C.byref(drawn))
        if n < 0:
            raise ValueError("oracle distributed render refused its arguments")
        return {"rgb": rgb, "ids": ids, "fimg": fimg, "rays": n, "drawn": drawn.value}

    def pixel_secondary_rays(self, frame, x, y):
        """(primary hit id, ogn, dir, tmax) of the secondary rays pixel
        (x, y) of the frame spawns: its AO rays for an AO frame, else one
        shadow ray per light (ro_pixel_secondary_rays)."""
        cam = make_camera(frame["camera"])
        ao = frame.get("ao")
        lights = frame.get("lights") or []
        ls = make_lights(lights)
        n_max = max(1, ao["samples"] if ao else len(lights))
        ogn = np.zeros((n_max, 3), np.float32)
        dirs = np.zeros((n_max, 3), np.float32)
        tmax = np.zeros(n_max, np.float32)
        hid = np.zeros(1, np.int32)
        n = self.lib["ro_pixel_secondary_rays"](self.h, C.byref(cam), ls, 0 if ao else len(lights),
                                                ao["samples"] if ao else 0, ao["dist"] if ao else 0.0,
                                                ao["seed"] if ao else 0, int(x), int(y), _p(hid, C.c_int32),
                                                _p(ogn, C.c_float), _p(dirs, C.c_float), _p(tmax, C.c_float))
        if n < 0:
            raise ValueError("bad pixel or frame")
        return int(hid[0]), ogn[:n], dirs[:n], tmax[:n]

    def render(self, frame, rows=None, threads=1, want_ids=False, want_float=False, want_occl=False):
        cam = make_camera(frame["camera"])
        W, H = cam.xres, cam.yres
        r0, r1 = (0, H) if rows is None else rows
        rgb = np.zeros((H, W, 3), np.uint8)
        ids = np.full((H, W), -2, np.int32) if want_ids else None
        occl = np.zeros((H, W), np.uint8) if want_occl else None
        fimg = np.zeros((H, W, 3), np.float32) if want_float else None
        mat = make_material(frame["material"])
        ao = frame.get("ao")
        if ao:
            cnt = np.zeros((H, W), np.int32)
            n = self.lib["ro_render_ao"](self.h, C.byref(cam), C.byref(mat), ao["samples"], ao["dist"], ao["seed"],
                                         r0, r1, threads, _p(rgb, C.c_uint8), _p(ids, C.c_int32), _p(cnt, C.c_int32))
            out = {"rgb": rgb, "ids": ids, "ao_count": cnt, "rays": n}
        else:
            ls = make_lights(frame["lights"])
            table = make_materials(frame["materials"]) if frame.get("materials") else None
            if table is not None:
                n = self.lib["ro_render_mt"](self.h, C.byref(cam), ls, len(frame["lights"]), table, len(table), r0, r1,
                                             threads, _p(rgb, C.c_uint8), _p(ids, C.c_int32), _p(occl, C.c_uint8),
                                             _p(fimg, C.c_float))
            else:
                n = self.lib["ro_render"](self.h, C.byref(cam), ls, len(frame["lights"]), C.byref(mat), r0, r1,
                                          threads, _p(rgb, C.c_uint8), _p(ids, C.c_int32), _p(occl, C.c_uint8),
                                          _p(fimg, C.c_float))
            out = {"rgb": rgb, "ids": ids, "occl": occl, "fimg": fimg, "rays": n}
        if n < 0:
            raise RuntimeError("oracle render failed")
        return out


class RefScene(_SceneBase):
    """The reference's own bvh + ray_tracer behind the harness (x86 only)."""
    prefix = "rref_"

    def __init__(self, scene, material, soft=False, diffuse=False):
        """material: one material dict, or a list of them indexed by
        scene["mat_of_tri"] (one coloured_mapper_shader per entry).  soft:
        the reference built with soft shadows (ref_soft_lib); diffuse: with
        soft shadows and diffuse reflections (ref_diffuse_lib)."""
        self.lib = ref_diffuse_lib() if diffuse else ref_soft_lib() if soft else ref_lib()
        v, t, a, f = _scene_arrays(scene)
        self._keep = (v, t, a, f)
        if isinstance(material, (list, tuple)):
            self.mat = make_materials(material)
            mt = scene.get("mat_of_tri")
            mt = None if mt is None else np.ascontiguousarray(mt, np.int32)
            self._keep = self._keep + (mt,)
            self.h = self.lib["rref_scene_create_mt"](_p(v, C.c_float), v.shape[0], _p(t, C.c_int32), t.shape[0],
                                                      _p(a, C.c_float), _p(f, C.c_uint32), self.mat, len(self.mat),
                                                      _p(mt, C.c_int32))
        else:
            self.mat = make_material(material)
            self.h = self.lib["rref_scene_create"](_p(v, C.c_float), v.shape[0], _p(t, C.c_int32), t.shape[0],
                                                   _p(a, C.c_float), _p(f, C.c_uint32), C.byref(self.mat))
        self.build_seconds = self.lib["rref_scene_build"](self.h)

    def render(self, frame, aa=(1, 1), tone=None):
        """ray_tracer + clip_image_to_rgb; aa = (x_a_res, y_a_res) rays per
        output pixel along x and y (the camera's anti-aliasing factors);
        tone: a tone-map dict (camera::tone_map + gamma_correct before the
        clip) or None."""
        cam = make_camera(frame["camera"])
        rgb = np.zeros((cam.yres, cam.xres, 3), np.uint8)
        ls = make_lights(frame["lights"])
        if tone is None:
            secs = self.lib["rref_render_aa"](self.h, C.byref(cam), int(aa[0]), int(aa[1]), ls,
                                              len(frame["lights"]), _p(rgb, C.c_uint8))
        else:
            tm = make_tone_map(tone)
            secs = self.lib["rref_render_tone_mapped"](self.h, C.byref(cam), int(aa[0]), int(aa[1]), ls,
                                                       len(frame["lights"]), C.byref(tm), _p(rgb, C.c_uint8))
        return {"rgb": rgb, "seconds": secs}


def supersampled(frame, aa_x, aa_y):
    """The frame with aa_x * aa_y camera rays per output pixel: the camera
    grid the reference traces for x_a_res / y_a_res (camera.h:55-62)."""
    f = dict(frame)
    cam = dict(frame["camera"])
    cam["xres"] = cam["xres"] * aa_x
    cam["yres"] = cam["yres"] * aa_y
    f["camera"] = cam
    return f


def downsample_rgb8(fimg, aa_x, aa_y):
    """camera::clip_image_to_rgb (camera.h:289-319) on a supersampled float
    image (row = y): per output pixel the samples are summed in binary32,
    a_x outer and a_y inner, starting from 0, divided by their count,
    clamped to [0, 255] and truncated."""
    fimg = np.asarray(fimg, np.float32)
    H, W = fimg.shape[0] // aa_y, fimg.shape[1] // aa_x
    acc = np.zeros((H, W, 3), np.float32)
    for a_x in range(aa_x):
        for a_y in range(aa_y):
            acc = acc + fimg[a_y::aa_y, a_x::aa_x, :][:H, :W]
    v = acc / np.float32(aa_x * aa_y)
    return np.minimum(np.float32(255.0), np.maximum(np.float32(0.0), v)).astype(np.uint8)


def render_aa(scene_obj, frame, aa_x, aa_y):
    """Anti-aliased frame by the restatement: the supersampled float image of
    OracleScene.render, then downsample_rgb8."""
    out = scene_obj.render(supersampled(frame, aa_x, aa_y), want_float=True)
    return downsample_rgb8(out["fimg"], aa_x, aa_y)


def ref_tone_map_image(fimg, camera, tone, aa=(1, 1)):
    """The reference's camera::tone_map + gamma_correct + clip_image_to_rgb
    on a given supersampled float frame (rows = y)."""
    cam = make_camera(camera)
    img = np.ascontiguousarray(fimg, np.float32)
    rgb = np.zeros((cam.yres, cam.xres, 3), np.uint8)
    ref_lib()["rref_tone_map_image"](C.byref(cam), int(aa[0]), int(aa[1]), _p(img, C.c_float),
                                     C.byref(make_tone_map(tone, camera)), _p(rgb, C.c_uint8))
    return rgb


def ref_parse_and_render(path, kind, frame):
    """The reference's own parser (its default phong materials) followed by
    its bvh, ray_tracer and clip_image_to_rgb on frame's camera and lights."""
    cam = make_camera(frame["camera"])
    rgb = np.zeros((cam.yres, cam.xres, 3), np.uint8)
    ls = make_lights(frame["lights"])
    n = ref_lib()["rref_parse_and_render"](str(path).encode(), kind, C.byref(cam), ls, len(frame["lights"]),
                                           _p(rgb, C.c_uint8))
    if n < 0:
        raise OSError(f"cannot open {path}")
    return rgb


def ref_parse_mesh(path, kind):
    """The reference's own OFF (kind 1) / PLY (kind 2) parser on a file:
    (triangles as an (n, 9) float32 array of a, b, c vertices in
    primitive_store order, number of materials it made)."""
    lib = ref_lib()
    nmat = C.c_int32()
    n = lib["rref_parse_mesh"](str(path).encode(), kind, None, 0, C.byref(nmat))
    if n < 0:
        raise OSError(f"cannot open {path}")
    out = np.zeros((max(n, 1), 9), np.float32)
    lib["rref_parse_mesh"](str(path).encode(), kind, _p(out, C.c_float), n, C.byref(nmat))
    return out[:n], nmat.value


def tone_map_frame(fimg, tone, camera=None):
    """camera::tone_map + gamma_correct restated (ro_tone_map_frame) on a
    copy of a float frame (rows = y, 0..255 colours); camera: the frame's
    camera dict (needed by the histogram modes)."""
    img = np.array(fimg, np.float32, order="C", copy=True)
    tm = make_tone_map(tone, camera)
    if oracle_lib()["ro_tone_map_frame"](_p(img, C.c_float), img.shape[1], img.shape[0], C.byref(tm)) != 0:
        raise ValueError("unsupported tone-mapping mode")
    return img


def render_tone_mapped(scene_obj, frame, tone, aa=(1, 1)):
    """Tone-mapped (anti-aliased) frame by the restatement: the supersampled
    float image, tone_map_frame, then downsample_rgb8."""
    out = scene_obj.render(supersampled(frame, *aa), want_float=True)
    return downsample_rgb8(tone_map_frame(out["fimg"], tone, frame["camera"]), *aa)


def camera_rays(cam_dict, x0=0, y0=0, w=None, h=None, lib=None):
    lib = lib or oracle_lib()
    cam = make_camera(cam_dict)
    w = cam.xres if w is None else w
    h = cam.yres if h is None else h
    ogn = np.empty((w * h, 3), np.float32)
    dirs = np.empty((w * h, 3), np.float32)
    pre = "rref_" if lib is _ref else "ro_"
    lib[pre + "camera_rays"](C.byref(cam), x0, y0, w, h, _p(ogn, C.c_float), _p(dirs, C.c_float))
    return ogn, dirs


def morton(x, y, z, xm, ym, zm, lib=None):
    lib = lib or oracle_lib()
    pre = "rref_" if lib is _ref else "ro_"
    return lib[pre + "morton_code"](x, y, z, xm, ym, zm) & 0xFFFFFFFF


def ao_rays(hit_point, geo_normal, pixel, nsamples, seed):
    lib = oracle_lib()
    hp = np.ascontiguousarray(hit_point, np.float32)
    gn = np.ascontiguousarray(geo_normal, np.float32)
    ogn = np.empty((nsamples, 3), np.float32)
    dirs = np.empty((nsamples, 3), np.float32)
    lib["ro_ao_rays"](_p(hp, C.c_float), _p(gn, C.c_float), pixel, nsamples, seed, _p(ogn, C.c_float),
                      _p(dirs, C.c_float))
    return ogn, dirs


def ref_random(start, n):
    """n numbers of the reference's random stream from position start (the
    restatement, ro_ref_random)."""
    out = np.empty(n, np.float32)
    oracle_lib()["ro_ref_random"](int(start), int(n), _p(out, C.c_float))
    return out


TREE_ROOT = 0x6A09E667F3BCC909


def pixel_stream(seed, pixel, node, k):
    """Number k that tree node `node` of pixel `pixel` draws (ro_pixel_stream)."""
    return oracle_lib()["ro_pixel_stream"](int(seed), int(pixel), int(node), int(k))


def tree_child(parent, set_, index):
    """The tree node of ray `index` of a node's reflection (0) or refraction
    (1) set (ro_tree_child)."""
    return oracle_lib()["ro_tree_child"](int(parent), int(set_), int(index))


def area_light_rays(ntris, n):
    """(rays made, rays per triangle) of a triangle-defined light of ntris
    triangles asked for n rays (ro_area_light_rays)."""
    cnt = np.zeros(max(1, int(ntris)), np.int32)
    made = oracle_lib()["ro_area_light_rays"](int(ntris), int(n), _p(cnt, C.c_int32))
    return made, cnt[:int(ntris)]


def philox(ctr, key0, key1):
    lib = oracle_lib()
    c = np.ascontiguousarray(ctr, np.uint32)
    o = np.empty(4, np.uint32)
    lib["ro_philox4x32"](_p(c, C.c_uint32), key0, key1, _p(o, C.c_uint32))
    return o
