"""GPU parity of the differentiable render and its adjoint (bh_render_adjoint)
against the FP64 oracle (bh_oracle_smooth.cc): the image against the oracle's
render, the gradient against the oracle's dual-number gradient and against
FP64 central finite differences of the oracle's FP64 loss."""
import ctypes as C
import math

import numpy as np
import pytest

from blackhole_8_gb300 import capi

from helpers import adjoint_case, adjoint_thetas, fd_protocol

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _run(renderer, scenes, theta, targets, options, image=True, pixel_grad=True):
    """bh_render_adjoint over mirror scenes; returns (results, images,
    per-pixel gradients) as numpy."""
    cs = renderer.c_scenes(scenes)
    n = len(scenes)
    frames = (capi.AdjointFrame * n)()
    keep = []
    imgs, grads = [], []
    for i, sc in enumerate(scenes):
        h, w = sc.camera.height(), sc.camera.width()
        tg = None
        if targets is not None and targets[i] is not None:
            tg = torch.from_numpy(np.ascontiguousarray(targets[i], dtype=np.float32)).cuda()
        im = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda") if image else None
        gr = torch.zeros((h, w, capi.GRAD_COUNT), dtype=torch.float32, device="cuda") if pixel_grad else None
        frames[i].target = tg.data_ptr() if tg is not None else None
        frames[i].image = im.data_ptr() if im is not None else None
        frames[i].pixel_grad = gr.data_ptr() if gr is not None else None
        keep += [tg, im, gr]
        imgs.append(im)
        grads.append(gr)
    torch.cuda.synchronize()
    res = renderer.render_adjoint(cs, frames, theta, options)
    return (res, [None if x is None else x.cpu().numpy() for x in imgs],
            [None if x is None else x.cpu().numpy() for x in grads])


def test_forward_matches_oracle_image(renderer):
    from oracle import oracle
    sc, th0, tt, _ = adjoint_case(96, 64)
    # images are float32: FP64 agrees to float rounding
    for prec, tol in ((capi.PRECISION_FP64, 1e-7), (capi.PRECISION_MIXED, 2e-3), (capi.PRECISION_FP32, 2e-2)):
        res, imgs, _ = _run(renderer, [sc], tt[None], None, capi.adjoint_options(precision=prec), pixel_grad=False)
        ref, _, _ = oracle.smooth_render(sc, tt)
        err = np.abs(imgs[0] - ref)
        assert np.quantile(err, 0.999) <= tol, (prec, np.quantile(err, 0.999))
        assert res[0].loss == 0.0 and res[0].steps > 0


def test_fp64_adjoint_matches_dual(renderer):
    """Reverse mode (FP64) == forward-mode dual numbers (FP64), per pixel and
    summed, at a theta away from the scene's own."""
    from oracle import oracle
    sc, th0, tt, target = adjoint_case(96, 64)
    th = th0 + 0.5 * (tt - th0)
    th[capi.GRAD_ROLL] += 0.01
    th[capi.GRAD_CAM_Y] -= 0.2
    res, imgs, grads = _run(renderer, [sc], th[None], [target], capi.adjoint_options(precision=capi.PRECISION_FP64))
    g_dual = oracle.smooth_grad(sc, target, th)
    img_ref, l_ref, _ = oracle.smooth_render(sc, th, target)
    assert abs(res[0].loss - l_ref.sum() / target.size) <= 1e-9 * max(1.0, l_ref.sum())
    g = grads[0]
    for i in range(capi.GRAD_COUNT):
        scale = np.abs(g_dual[..., i]).max()
        np.testing.assert_allclose(g[..., i], g_dual[..., i], rtol=1e-4, atol=1e-5 * scale,
                                   err_msg=capi.GRAD_NAMES[i])
        total = g_dual[..., i].sum() / target.size
        assert abs(res[0].grad[i] - total) <= 1e-5 * np.abs(g_dual[..., i]).sum() / target.size, capi.GRAD_NAMES[i]


def test_mixed_adjoint_matches_dual(renderer):
    from oracle import oracle
    sc, th0, tt, target = adjoint_case(128, 128)
    res, _, grads = _run(renderer, [sc], th0[None], [target], capi.adjoint_options())
    g_dual = oracle.smooth_grad(sc, target, th0)
    assert res[0].band_rays > 0
    g_ref = g_dual.reshape(-1, capi.GRAD_COUNT).sum(0) / target.size
    g = np.array(res[0].grad)
    assert np.linalg.norm(g - g_ref) <= 1e-3 * np.linalg.norm(g_ref)
    for i in range(capi.GRAD_COUNT):
        l1 = np.abs(g_dual[..., i]).sum() / target.size
        assert abs(g[i] - g_ref[i]) <= 1e-3 * l1, (capi.GRAD_NAMES[i], g[i], g_ref[i], l1)


def test_adjoint_passes_finite_difference_check(renderer):
    """The library's gradient against FP64 central differences of the FP64
    loss (the oracle's), h = 1e-5 with Richardson from h/2 and a resolution
    check at h/4, over the pixels where the differences are resolved and the
    ray's structure does not change: FP64 each parameter to 1e-3; MIXED the
    gradient vector to 1e-3 and each parameter to 1e-3 of its scale."""
    from oracle import oracle
    sc, th0, tt, target = adjoint_case(64, 48)
    _, _, g64 = _run(renderer, [sc], th0[None], [target], capi.adjoint_options(precision=capi.PRECISION_FP64))
    _, _, gmx = _run(renderer, [sc], th0[None], [target], capi.adjoint_options())
    loss_at = lambda th: oracle.smooth_render(sc, th, target)[1]
    sig_at = lambda th: oracle.smooth_render(sc, th, target)[2]
    fd_v, mx_v = [], []
    for i in range(capi.GRAD_COUNT):
        rich, ok = fd_protocol(loss_at, th0, i, signature_at=sig_at)
        assert ok.mean() > 0.9, (capi.GRAD_NAMES[i], ok.mean())
        fd, ad = rich[ok].sum(), g64[0][..., i][ok].sum()
        assert abs(fd - ad) <= 1e-3 * abs(fd), (capi.GRAD_NAMES[i], fd, ad)
        mx = gmx[0][..., i][ok].sum()
        assert abs(fd - mx) <= 1e-3 * np.abs(rich[ok]).sum(), (capi.GRAD_NAMES[i], fd, mx)
        fd_v.append(fd)
        mx_v.append(mx)
    fd_v, mx_v = np.array(fd_v), np.array(mx_v)
    assert np.linalg.norm(mx_v - fd_v) <= 1e-3 * np.linalg.norm(fd_v)


def test_precisions_and_band(renderer):
    sc, th0, tt, target = adjoint_case(64, 64)
    r64, _, g64 = _run(renderer, [sc], None, [target], capi.adjoint_options(precision=capi.PRECISION_FP64))
    r32, _, g32 = _run(renderer, [sc], None, [target], capi.adjoint_options(precision=capi.PRECISION_FP32))
    rm0, _, _ = _run(renderer, [sc], None, [target], capi.adjoint_options(band=0.0))
    rmw, _, _ = _run(renderer, [sc], None, [target], capi.adjoint_options(band=1e3))
    assert np.isfinite(g32[0]).all() and np.isfinite(np.array(r32[0].grad)).all()
    assert rm0[0].band_rays == 0 and r64[0].band_rays == 0
    # every ray in the band: FP64-accurate forward with the texture filter in
    # FP32 (colours within ~1e-7 of the FP64 call's) and an FP32 reverse pass
    assert rmw[0].band_rays == 64 * 64
    g, g64 = np.array(rmw[0].grad), np.array(r64[0].grad)
    assert np.linalg.norm(g - g64) <= 5e-5 * np.linalg.norm(g64)
    assert abs(rmw[0].loss - r64[0].loss) <= 1e-6 * r64[0].loss


def test_batched_scenes_equal_single_calls(renderer):
    from blackhole_8_gb300 import scene as S
    a, th_a, tt_a, tg_a = adjoint_case(64, 48)
    b = S.single_scene(40, 72)
    th_b, tt_b = adjoint_thetas(b)
    from oracle import oracle
    tg_b = oracle.smooth_render(b, tt_b)[0].astype(np.float32)
    opts = capi.adjoint_options(precision=capi.PRECISION_FP64)
    both, _, _ = _run(renderer, [a, b], np.stack([th_a, th_b]), [tg_a, tg_b], opts, image=False, pixel_grad=False)
    one_a, _, _ = _run(renderer, [a], th_a[None], [tg_a], opts, image=False, pixel_grad=False)
    one_b, _, _ = _run(renderer, [b], th_b[None], [tg_b], opts, image=False, pixel_grad=False)
    for x, y in ((both[0], one_a[0]), (both[1], one_b[0])):
        assert abs(x.loss - y.loss) <= 1e-12 + 1e-9 * y.loss
        np.testing.assert_allclose(np.array(x.grad), np.array(y.grad), rtol=1e-6, atol=1e-12)
        assert x.steps == y.steps


def test_long_near_critical_rays_checkpointing(renderer):
    """Rays of 1000-2000 steps (20-30 checkpoints of 64 steps) within 1e-4 M of
    the critical impact parameter: FP64 adjoint == dual per pixel."""
    from oracle import oracle
    from blackhole_8_gb300 import scene as S
    sc = S.photon_ring_scene(24, fov_deg=2e-4)
    th0, tt = adjoint_thetas(sc)
    target = oracle.smooth_render(sc, tt, max_steps=12000)[0].astype(np.float32)
    opts = capi.adjoint_options(precision=capi.PRECISION_FP64, max_steps=12000)
    res, _, grads = _run(renderer, [sc], th0[None], [target], opts)
    assert res[0].steps / (24 * 24) > 1000
    g_dual = oracle.smooth_grad(sc, target, th0, max_steps=12000)
    scale = np.abs(g_dual).max()
    for i in range(capi.GRAD_COUNT):
        np.testing.assert_allclose(grads[0][..., i], g_dual[..., i], rtol=1e-4, atol=1e-6 * scale,
                                   err_msg=capi.GRAD_NAMES[i])


def test_torch_shim(renderer):
    from blackhole_8_gb300.torch_shim import render_loss
    sc, th0, tt, target = adjoint_case(48, 32)
    cs = renderer.c_scenes([sc])[0]
    tgt = torch.from_numpy(target).cuda()
    theta = torch.tensor(th0, dtype=torch.float64, requires_grad=True)
    opts = capi.adjoint_options(precision=capi.PRECISION_FP64)
    loss = render_loss(theta, renderer, cs, tgt, opts)
    loss.backward()
    ref, _, _ = _run(renderer, [sc], th0[None], [target], opts, image=False, pixel_grad=False)
    assert abs(loss.item() - ref[0].loss) <= 1e-12
    np.testing.assert_allclose(theta.grad.numpy(), np.array(ref[0].grad), rtol=1e-9)
    # one gradient-descent step on the pose lowers the loss
    with torch.no_grad():
        step = theta.clone()
        g = theta.grad.clone()
        g[capi.GRAD_MASS] = 0
        g[capi.GRAD_R_INNER] = 0
        g[capi.GRAD_R_OUTER] = 0
        step -= 1e-3 * g / g.norm()
    assert render_loss(step, renderer, cs, tgt, opts).item() < loss.item()


def test_invalid_arguments(renderer):
    sc, th0, tt, target = adjoint_case(16, 16)
    cs = renderer.c_scenes([sc])
    frames = (capi.AdjointFrame * 1)()
    lib = renderer.lib
    for kw, code in ((dict(step=0.5), capi.BH_ERR_INVALID_ARGUMENT),
                     (dict(checkpoint_every=32), capi.BH_ERR_UNSUPPORTED),
                     (dict(threads_per_block=256), capi.BH_ERR_UNSUPPORTED),
                     (dict(softness=-1.0), capi.BH_ERR_INVALID_ARGUMENT),
                     (dict(precision=7), capi.BH_ERR_INVALID_ARGUMENT)):
        o = capi.adjoint_options(**kw)
        assert lib.bh_render_adjoint(renderer.ctx, cs, 1, None, frames, C.byref(o), None) == code, kw
    bad = th0.copy()
    bad[3] = math.inf
    o = capi.adjoint_options()
    assert lib.bh_render_adjoint(renderer.ctx, cs, 1, bad.ctypes.data, frames, C.byref(o), None) == \
        capi.BH_ERR_INVALID_ARGUMENT
    assert b"theta" in lib.bh_last_error(renderer.ctx)
    far = th0.copy()
    far[capi.GRAD_CAM_X] = 1e4
    assert lib.bh_render_adjoint(renderer.ctx, cs, 1, far.ctypes.data, frames, C.byref(o), None) == \
        capi.BH_ERR_UNSUPPORTED
