"""Host-side checks that need no GPU: the shared library loads and exports
every entry point include/rtcore.h declares, argument validation returns
error codes, the ctypes mirrors of the ABI structs have the C sizes, the
workload generators are deterministic and have the configured sizes, and
the multi-process (replica) aggregation of bench.py works over gloo."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "rtcore.h")).read()
    return sorted(set(re.findall(r"^\s*(?:rt_status|const char \*|int32_t)\s*(rt_\w+)\s*\(", src, re.M)))


def test_library_exports_every_header_function(rtlib):
    names = header_functions()
    assert len(names) >= 25
    lib = C.CDLL(os.path.join(ROOT, "raptor_gb300", "_lib", "librtcore.so"))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes binding declares every one of them
    bound = {s[0] for s in rtlib.SIGNATURES}
    assert set(names) <= bound, set(names) - bound


def test_struct_sizes(rtlib):
    assert C.sizeof(rtlib.RtRay) == 32
    assert C.sizeof(rtlib.RtHit) == 16
    assert C.sizeof(rtlib.RtCamera) == 4 * (15 + 3) + 8
    assert C.sizeof(rtlib.RtLight) == 4 * 13
    assert C.sizeof(rtlib.RtMaterial) == 64
    assert C.sizeof(rtlib.RtLightShape) == 16
    assert C.sizeof(rtlib.RtSampling) == 32
    assert rtlib.RAY_DTYPE.itemsize == 32 and rtlib.HIT_DTYPE.itemsize == 16


def test_argument_validation_without_device(rtlib):
    L = rtlib.lib()
    assert rtlib.lib().rt_version() == 100
    assert L.rt_ctx_create(0, None) == -1
    assert L.rt_scene_upload(None, None, 0, None, 0, None, None) == -1
    assert L.rt_trace_closest(None, None, 0, None) == -1
    assert L.rt_render(None, None, None, 0, None, None, None, None) == -1
    assert L.rt_bvh_build(None, None) == -1
    assert L.rt_batch_set_jobs(None, None, 0) == -1
    assert L.rt_ctx_destroy(None) == 0
    assert L.rt_last_error_string() != b""


def test_context_without_gpu_reports_no_device(rtlib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert rtlib.lib().rt_ctx_create(0, C.byref(h)) == -7


def test_generators_deterministic_and_sized():
    from raptor_gb300 import scenes
    a, fa = scenes.icosphere_scene()
    b, fb = scenes.icosphere_scene()
    assert a["tris"].shape == (20482, 3) and a["verts"].shape == (10242 + 4, 3)
    for k in ("verts", "tris", "vattr"):
        assert np.array_equal(a[k], b[k])
    r = np.linalg.norm(a["verts"][:10242].astype(np.float64), axis=1)
    assert np.allclose(r, 1.0, atol=1e-6)
    # every sphere triangle faces outward
    v, t = a["verts"].astype(np.float64), a["tris"][:20480]
    n = np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]])
    assert ((n * v[t[:, 0]]).sum(1) > 0).all()
    s, f = scenes.terrain_scene(size_pow2=64, xres=64, yres=36)
    assert s["tris"].shape == (2 * 64 * 64, 3)
    assert np.isclose(s["verts"][:, 1].min(), 0.0) and np.isclose(s["verts"][:, 1].max(), 200.0)
    assert np.isclose(s["verts"][:, 0].max(), 1024.0)
    v50, t50, _ = scenes.displaced_sphere()
    assert t50.shape == (50000, 3)
    inst, _ = scenes.instances_scene(n_inst=10)
    assert inst["tris"].shape == (20000, 3)


def test_full_size_counts():
    from raptor_gb300 import scenes
    s, f = scenes.terrain_scene()
    assert s["tris"].shape[0] == 2097152 and f["camera"]["xres"] == 1920 and f["camera"]["yres"] == 1080
    i, fi = scenes.instances_scene()
    assert i["tris"].shape[0] == 4000000 and fi["ao"]["samples"] == 16 and fi["ao"]["dist"] == 5.0
    items = scenes.batched_scenes()
    assert len(items) == 64
    tri = np.array([sc["tris"].shape[0] for sc, _ in items])
    assert tri.min() >= 500 and tri.max() <= 600000
    assert {fr.get("ao", {}).get("samples", 0) for _, fr in items} == {0, 4}


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, ROOT)
    import bench
    t = bench.max_over_ranks(0.5 + rank, world, device="cpu")
    v = bench.aggregate_rate(1_000_000, t, world)
    out.put((rank, t, v))
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks_gloo():
    """bench.py on N GPUs: every rank renders its own replica; the whole-job
    value is all ranks' rays over the slowest rank's time."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in res:
        assert t == 1.5                       # max over ranks
        assert abs(v - 2 * 1_000_000 / 1.5 / 1e6) < 1e-9
