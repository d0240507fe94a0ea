"""The finite-difference check of tests/test_gpu_adjoint.py, checked on the
CPU: on the oracle's frame of the 50,000-triangle displaced icosphere
(256x256, the same hits and shadow bits as the CUDA forward up to ties),
the Richardson-extrapolated FP64 central differences of
F = sum_pix w . c_pix agree with the exact FP64 gradient of the same model
(torch autograd) to 1e-5 relative on all 200 vertices.  (A single central
difference is off by up to 1e-2 on these heavily cancelled sums, through
its O(h^2) truncation error, which is why the GPU test extrapolates.)"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_richardson_fd_is_exact_on_the_model(oracle):
    import test_gpu_adjoint as A
    from raptor_gb300 import scenes
    scene, tscene, frame = scenes.adjoint_scene()
    ref = oracle.OracleScene(scene).render(frame, want_ids=True, want_occl=True, want_float=True, threads=8)
    tgt = oracle.OracleScene(tscene).render(frame, want_float=True, threads=8)["fimg"]
    ids, occl = ref["ids"].reshape(-1), ref["occl"].reshape(-1)
    o, d = oracle.camera_rays(frame["camera"])
    hit = ids >= 0
    sgn, lit, spec, excluded = A.fp64_state(scene, frame, ids, o, d, hit)
    w = 2.0 * (ref["fimg"] - tgt).reshape(-1, 3).astype(np.float64)
    w[np.nonzero(hit)[0][excluded]] = 0.0
    V = torch.tensor(scene["verts"], dtype=torch.float64, requires_grad=True)
    C = torch.tensor(scene["vattr"], dtype=torch.float64, requires_grad=True)
    T = lambda a, dt=torch.float64: torch.tensor(a, dtype=dt)
    c = A.pixel_model(V, C, T(scene["tris"].astype(np.int64), torch.int64), T(ids[hit].astype(np.int64), torch.int64),
                      T(occl[hit].astype(np.float64)), T(o[hit].astype(np.float64)), T(d[hit].astype(np.float64)),
                      T(sgn), T(lit), T(spec, torch.bool), frame, torch)
    (T(w[hit]) * c).sum().backward()
    seen = np.unique(scene["tris"][ids[hit]].reshape(-1))
    picks = np.random.default_rng(4).choice(seen, 200, replace=False)
    fd_pos, fd_col = A.fd_vjp(scene, frame, ids, occl, o, d, w, picks)
    for fd, exact in ((fd_pos, V.grad.numpy()[picks]), (fd_col, C.grad.numpy()[picks])):
        rel = np.abs(fd - exact) / np.maximum(np.abs(exact), 1e-2 * np.sqrt((exact ** 2).mean()))
        assert rel.max() < 1e-5, rel.max()
