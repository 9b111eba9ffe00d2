"""Differentiable rendering: forward parity, adjoint vs FP64 gradient and FD, fitting.

* the GPU forward equals the oracle's float forward (same float operations);
* the adjoint's knot and voxel gradients match the oracle's FP64 analytic
  gradient to <= 1e-3 relative (L2 over all parameters);
* (the FP64 gradient itself is checked against central finite differences in
  tests/test_oracle_kat.py);
* torch.autograd through the C ABI gives the same gradients, and Adam
  lowers the loss.
"""

import numpy as np
import pytest

import hydrant_gb300 as hy
from hydrant_gb300 import fit
from oracle import oracle as orc
from tests._harness import view_array

pytestmark = pytest.mark.gpu

N = 24
W = H = 20


@pytest.fixture(scope="module")
def setup(ctx):
    torch = pytest.importorskip("torch")
    vol_true = hy.synth_blobs_f32(4, (N, N, N), 6)
    vol_init = hy.synth_blobs_f32(5, (N, N, N), 6)
    holder = hy.Volume(ctx, vol_true, N, 1)  # bbox [0,1]^3 for the camera helper
    views = fit.orbit_views(holder, 7, 3)
    holder.close()
    tf_true = fit.seeded_tf(9, 16)
    tf_init = np.full((16, 4), 0.5, np.float32)
    r = fit.DiffRenderer(ctx, N, views, W, H, 16, sample_rate=1.0, density=1.0, ckpt_k=8)
    return dict(torch=torch, vt=vol_true, vi=vol_init, views=views, tft=tf_true, tfi=tf_init, r=r)


def _va(views):
    return np.stack([view_array(v) for v in views])


def test_forward_matches_oracle(setup):
    torch = setup["torch"]
    r = setup["r"]
    img = r.forward(torch.from_numpy(setup["vi"]).cuda(), torch.from_numpy(setup["tft"]).cuda())
    torch.cuda.synchronize()
    ref = orc.diff_forward(setup["vi"], setup["tft"], _va(setup["views"]), W, H)
    got = img.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-6
    assert got[..., 3].max() > 0.05


def test_adjoint_matches_fp64_gradient(setup):
    torch = setup["torch"]
    r = setup["r"]
    va = _va(setup["views"])
    _, target, _, _ = orc.diff_loss_grad64(setup["vt"], setup["tft"], va, W, H, grad=False)
    # a non-uniform TF: with the uniform initial one the image does not depend
    # on the voxels at all (dTF/ds = 0) and the voxel gradient is exactly 0
    tf_eval = np.clip(setup["tft"] * 0.8 + 0.1, 0, 1).astype(np.float32)
    loss64, img64, dv64, dt64 = orc.diff_loss_grad64(setup["vi"], tf_eval, va, W, H, target)
    assert np.linalg.norm(dv64) > 0 and np.linalg.norm(dt64) > 0
    vol = torch.from_numpy(setup["vi"]).cuda()
    tf = torch.from_numpy(tf_eval).cuda()
    img = r.forward(vol, tf)
    g = 2.0 * (img - torch.from_numpy(target.astype(np.float32)).cuda())
    dv, dt = r.backward(vol, tf, g.contiguous())
    torch.cuda.synchronize()
    dv, dt = dv.cpu().numpy().astype(np.float64), dt.cpu().numpy().astype(np.float64)
    rel_t = np.linalg.norm(dt - dt64) / np.linalg.norm(dt64)
    rel_v = np.linalg.norm(dv - dv64) / np.linalg.norm(dv64)
    assert rel_t <= 1e-3, rel_t
    assert rel_v <= 1e-3, rel_v


def test_autograd_and_adam(ctx, setup):
    torch = setup["torch"]
    res = fit.fit(ctx, setup["vt"], setup["vi"], setup["views"], W, H, setup["tft"], setup["tfi"],
                  steps=30, ckpt_k=8, lr_tf=2e-2, lr_vol=1e-2)
    assert res.losses[-1] < 0.5 * res.losses[0], res.losses[::5]
    # autograd gradients equal the direct backward call
    r = setup["r"]
    vol = torch.from_numpy(setup["vi"]).cuda().requires_grad_(True)
    tf = torch.from_numpy(setup["tfi"]).cuda().requires_grad_(True)
    img = fit.render(vol, tf, r)
    (img ** 2).sum().backward()
    dv, dt = r.backward(vol.detach(), tf.detach(), (2 * img).detach().contiguous())
    torch.cuda.synchronize()
    assert torch.allclose(vol.grad, dv, rtol=1e-4, atol=1e-5 * float(dv.abs().max()))
    assert torch.allclose(tf.grad, dt, rtol=1e-4, atol=1e-5 * float(dt.abs().max()))


@pytest.mark.parametrize("k", [4, 5, 1, 64])
def test_checkpoint_interval_does_not_change_gradients(ctx, setup, k):
    """The image does not depend on K; the gradients agree to 1e-4 relative:
    the adjoint recomputes each sample position from its segment's
    checkpoint in one rounding per axis, so positions (and the trilinear
    weights at them) differ from the forward's running sum by a few ulps
    that grow with the segment length, and the order of atomics between
    rays differs."""
    torch = setup["torch"]
    vol = torch.from_numpy(setup["vi"]).cuda()
    tf = torch.from_numpy(np.clip(setup["tft"] * 0.8 + 0.1, 0, 1).astype(np.float32)).cuda()
    out = []
    for kk in (8, k):
        r = fit.DiffRenderer(ctx, N, setup["views"], W, H, 16, sample_rate=1.0, density=1.0,
                             ckpt_k=kk)
        img = r.forward(vol, tf)
        g = torch.linspace(-1, 1, img.numel(), device="cuda").reshape(img.shape)
        dv, dt = r.backward(vol, tf, g)
        torch.cuda.synchronize()
        out.append((img.cpu().numpy(), dv.cpu().numpy(), dt.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0])
    for a, b in ((out[0][1], out[1][1]), (out[0][2], out[1][2])):
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(a), np.linalg.norm(a - b)


def test_adjoint_matches_finite_differences_at_k32(ctx):
    """The configuration's checkpoint interval (K = 32) on a mid-size case
    (64^3 f32, 4 views of 96^2, 32 knots): the adjoint's gradient of the mean
    squared image error against central finite differences (eps 1e-3, loss in
    float64) on the largest knot and voxel gradients, within 1e-3 relative
    in L2 over the checked set and 3e-3 for any one of them (the difference
    quotient carries the f32 rounding of the images)."""
    torch = pytest.importorskip("torch")
    n, res, ntf = 64, 96, 32
    vt = hy.synth_blobs_f32(4, (n, n, n), 12)
    vi = hy.synth_blobs_f32(5, (n, n, n), 12)
    holder = hy.Volume(ctx, vt, n, 1)
    views = fit.orbit_views(holder, 4, 4)
    holder.close()
    tft = fit.seeded_tf(4, ntf)
    r = fit.DiffRenderer(ctx, n, views, res, res, ntf, ckpt_k=32)
    target = r.forward(torch.from_numpy(vt).cuda(), torch.from_numpy(tft).cuda(), keep=False).clone()
    vol = torch.from_numpy(vi).cuda()
    tf = torch.from_numpy(np.clip(tft * 0.8 + 0.1, 0, 1).astype(np.float32)).cuda()
    img = r.forward(vol, tf)
    g = (2.0 / img.numel()) * (img - target)
    dv, dt = r.backward(vol, tf, g.contiguous())
    torch.cuda.synchronize()

    def loss(v, t):
        im = r.forward(v, t, keep=False)
        torch.cuda.synchronize()
        return float(((im.double() - target.double()) ** 2).mean())

    eps, pairs = 1e-3, []
    for grad, base, is_tf in ((dt, tf, True), (dv, vol, False)):
        for idx in torch.topk(grad.reshape(-1).abs(), 4).indices.tolist():
            p, m = base.clone(), base.clone()
            p.view(-1)[idx] += eps
            m.view(-1)[idx] -= eps
            fd = (loss(vol, p) - loss(vol, m)) if is_tf else (loss(p, tf) - loss(m, tf))
            pairs.append((float(grad.reshape(-1)[idx]), fd / (2 * eps)))
    a = np.array([x for x, _ in pairs])
    f = np.array([y for _, y in pairs])
    assert np.linalg.norm(a - f) <= 1e-3 * np.linalg.norm(f), (a, f)
    assert np.max(np.abs(a - f) / np.abs(f)) <= 3e-3, (a, f)
