"""Path-replay adjoint on the GPU (e8g_forward / e8g_backward): gradients of an L2 image loss
with respect to per-material albedo and GGX roughness, checked against central finite
differences with common random numbers, against the oracle's FP64 restatement of the same
gradient, and timed against the forward render."""
import ctypes as C

import numpy as np
import pytest

import oracle_bind as ob
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.core import default_params

pytestmark = pytest.mark.gpu


def perturbed(mats, seed=3, sigma=0.05):
    rng = np.random.default_rng(seed)
    out = []
    for m in mats:
        q = abi.Material.from_buffer_copy(m)
        if q.type in (abi.MAT_OREN_NAYAR, abi.MAT_COOK_TORR):
            q.albedo[:] = list(np.clip(np.array(list(m.albedo)) + rng.normal(0, sigma, 3), 0.05, 0.95))
        if q.type == abi.MAT_COOK_TORR:
            q.roughness = float(np.clip(m.roughness + rng.normal(0, sigma), 0.05, 1.0))
        out.append(q)
    return out


def loss_and_grad(img, target):
    d = img[..., :3].astype(np.float64) - target[..., :3]
    return float(np.sum(d * d)), (2 * d).astype(np.float32)


def setup(ctx, w, h, spp):
    sc = S.displaced_icosphere(level=4, seed=7, num_materials=16, width=w, height=h)
    ctx.upload(sc)
    base = sc.material_list()
    p = default_params(abi.MODE_MIS, w, h, spp, seed=11, max_depth=6, rr_start=3)
    ctx.set_materials(perturbed(base))
    target = ctx.render(p)
    ctx.set_materials(base)
    return sc, base, p, target


def render_loss(ctx, mats, p, target):
    ctx.set_materials(mats)
    return loss_and_grad(ctx.render(p), target)[0]


def image_from_paths(ctx, p):
    """The image as the float64 mean of its per-path radiance (e8g_render_paths): free of the
    accumulation-order rounding of atomics, so finite differences of tiny loss changes are exact
    up to the paths themselves."""
    w, h, spp = p.width, p.height, p.spp
    px = np.repeat(np.arange(w * h, dtype=np.uint32), spp)
    smp = np.tile(np.arange(spp, dtype=np.uint32), w * h)
    rad = ctx.render_paths(p, px, smp).astype(np.float64).reshape(h, w, spp, 3)
    return rad.mean(axis=2)


def path_loss(ctx, mats, p, target):
    ctx.set_materials(mats)
    d = image_from_paths(ctx, p) - target[..., :3]
    return float(np.sum(d * d))


def test_albedo_gradients_match_finite_differences(ctx):
    """Albedo does not move the sampling, so central differences with common random numbers and
    the replayed gradient agree path for path: within 1% on the eight leading components."""
    sc, base, p, target = setup(ctx, 64, 48, 32)
    ctx.forward(p)
    img = image_from_paths(ctx, p)
    dl = (2 * (img - target[..., :3])).astype(np.float32)
    da, dr = ctx.backward(dl)
    h = 1e-3
    checked = 0
    for m in range(16):
        for c in range(3):
            if abs(da[m, c]) < 1e-3 * np.abs(da).max():
                continue
            plus = [abi.Material.from_buffer_copy(x) for x in base]
            minus = [abi.Material.from_buffer_copy(x) for x in base]
            plus[m].albedo[c] += h
            minus[m].albedo[c] -= h
            fd = (path_loss(ctx, plus, p, target) - path_loss(ctx, minus, p, target)) / (2 * h)
            assert abs(fd - da[m, c]) <= 0.01 * abs(fd) + 1e-6, (m, c, fd, da[m, c])
            checked += 1
            if checked >= 8:
                break
        if checked >= 8:
            break
    ctx.set_materials(base)
    assert checked >= 4


def test_roughness_gradients_match_finite_differences(ctx):
    """Roughness moves the sampled GGX directions, so CRN finite differences and the replayed
    gradient (sampling held fixed) agree in expectation only: 96x72 pixels at 4096 spp (28M paths
    per render), the two largest gradients, within 3%."""
    sc, base, p, target = setup(ctx, 96, 72, 4096)
    img = ctx.forward(p)
    _, dl = loss_and_grad(img, target)
    da, dr = ctx.backward(dl)
    order = np.argsort(-np.abs(dr))[:2]
    h = 1e-3
    for m in order:
        plus = [abi.Material.from_buffer_copy(x) for x in base]
        minus = [abi.Material.from_buffer_copy(x) for x in base]
        plus[m].roughness += h
        minus[m].roughness -= h
        fd = (render_loss(ctx, plus, p, target) - render_loss(ctx, minus, p, target)) / (2 * h)
        assert abs(fd - dr[m]) <= 0.03 * abs(fd), (m, fd, dr[m])
    ctx.set_materials(base)


def test_gradients_match_fp64_oracle(ctx):
    w, h, spp = 24, 16, 4
    sc, base, p, target = setup(ctx, w, h, spp)
    img = ctx.forward(p)
    _, dl = loss_and_grad(img, target)
    da, dr = ctx.backward(dl)
    osc = ob.OracleScene(sc)
    nm = len(base)
    a64 = np.zeros(nm * 3)
    r64 = np.zeros(nm)
    rgb = np.zeros(3)
    pol = ob.OPolicy(6, 3, 0.5, 8)
    for px in range(w * h):
        wgt = (dl[px // w, px % w] / spp).astype(np.float32)
        for s in range(spp):
            ob.oracle().o_path_gradient_f64(osc.h, 11, C.byref(pol), w, h, px, s, ob.ptr(wgt), ob.ptr(a64),
                                            ob.ptr(r64), ob.ptr(rgb))
    a64 = a64.reshape(nm, 3)
    err_a = np.linalg.norm(da - a64) / np.linalg.norm(a64)
    err_r = np.linalg.norm(dr - r64) / max(np.linalg.norm(r64), 1e-12)
    assert err_a < 1e-2 and err_r < 1e-2, (err_a, err_r)


def test_adjoint_costs_at_most_three_forwards(ctx):
    sc = S.displaced_icosphere(level=6, seed=1, num_materials=256, width=256, height=256)
    ctx.upload(sc)
    p = default_params(abi.MODE_MIS, 256, 256, 16, seed=1, max_depth=6, rr_start=3)
    for _ in range(2):
        img = ctx.forward(p)
        fwd = ctx.stats()["ms"]
        ctx.backward(np.ones((256, 256, 3), np.float32))
        bwd = ctx.stats()["ms"]
    assert bwd <= 3.0 * fwd, (fwd, bwd)


def test_set_materials_roundtrip(ctx):
    sc = S.cornell(32, 32)
    ctx.upload(sc)
    p = default_params(abi.MODE_MIS, 32, 32, 4, seed=2)
    a = ctx.render(p)
    mats = sc.material_list()
    changed = [abi.Material.from_buffer_copy(m) for m in mats]
    changed[0].albedo[:] = [0.1, 0.1, 0.1]
    ctx.set_materials(changed)
    b = ctx.render(p)
    assert not np.allclose(a, b)
    ctx.set_materials(mats)
    c = ctx.render(p)
    assert np.allclose(a, c, rtol=1e-5, atol=1e-6)
    from x3dcore2_gb300.abi import E8GError
    with pytest.raises(E8GError, match="INVALID_ARG"):
        ctx.set_materials(mats[:2])


def test_backward_needs_forward(lib):
    from x3dcore2_gb300.abi import E8GError
    from x3dcore2_gb300.core import Context
    with Context(0) as c:
        c.upload(S.cornell(16, 16))
        with pytest.raises(E8GError, match="INVALID_ARG"):
            c.backward(np.zeros((16, 16, 3), np.float32))
        with pytest.raises(E8GError, match="INVALID_ARG"):  # the adjoint replays MIS + Philox paths
            c.forward(default_params(abi.MODE_REF_LT1, 16, 16, 1))


def test_autograd_function_gives_the_adjoints_gradients(ctx):
    """x3dcore2_gb300.autograd.render: torch's backward through the differentiable render gives
    e8g_backward's gradients of the same loss, and a second render on the context before the
    first graph's backward is refused."""
    import torch
    from x3dcore2_gb300 import autograd as AG
    sc, base, p, target = setup(ctx, 32, 24, 8)
    albedo = torch.tensor([list(m.albedo) for m in base], dtype=torch.float32, requires_grad=True)
    rough = torch.tensor([m.roughness for m in base], dtype=torch.float32, requires_grad=True)
    img = AG.render(ctx, p, albedo, rough)
    assert img.shape == (24, 32, 3)
    loss = ((img - torch.from_numpy(target[..., :3])) ** 2).sum()
    loss.backward()
    ctx.set_materials(base)
    ref = ctx.forward(p)
    # pixels sum their samples with atomics: the same render up to the order of those sums
    np.testing.assert_allclose(ref[..., :3], img.detach().numpy(), rtol=1e-5, atol=1e-6)
    _, dl = loss_and_grad(ref, target)
    da, dr = ctx.backward(dl)
    assert np.abs(da).max() > 0 and np.abs(dr).max() > 0
    np.testing.assert_allclose(albedo.grad.numpy(), da, rtol=1e-3, atol=1e-4 * np.abs(da).max())
    np.testing.assert_allclose(rough.grad.numpy(), dr, rtol=1e-3, atol=1e-4 * np.abs(dr).max())
    first = AG.render(ctx, p, albedo.detach().requires_grad_(), rough.detach().requires_grad_())
    AG.render(ctx, p, albedo.detach().requires_grad_(), rough.detach().requires_grad_())
    with pytest.raises(RuntimeError, match="another differentiable render"):
        first.sum().backward()
