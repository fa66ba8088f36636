"""Host logic of the torch.autograd binding (x3dcore2_gb300.autograd) against a fake context:
which materials take the tensors' values, how the image and the gradients travel, and the
refusal of a backward whose forward is no longer the context's last one. The GPU test in
test_gpu_adjoint.py checks the same binding against e8g_backward."""
import numpy as np
import pytest
import torch

from x3dcore2_gb300 import abi
from x3dcore2_gb300 import autograd as AG


def material(kind, albedo, rough):
    m = abi.Material()
    m.type = kind
    m.albedo[:] = albedo
    m.roughness = rough
    return m


class FakeCtx:
    def __init__(self, base):
        self.base = base
        self.set = None
        self.grad_in = None

    def set_materials(self, mats):
        self.set = [abi.Material.from_buffer_copy(m) for m in mats]

    def forward(self, params):
        img = np.zeros((params.height, params.width, 4), np.float32)
        img[..., 0] = self.set[1].albedo[0]
        img[..., 3] = 1.0
        return img

    def backward(self, g):
        self.grad_in = g.copy()
        nm = len(self.base)
        return np.full((nm, 3), 2.0, np.float32), np.arange(nm, dtype=np.float32)


def params(w, h):
    p = abi.RenderParams()
    p.width, p.height = w, h
    return p


def test_materials_images_and_gradients_travel():
    base = [material(abi.MAT_FAIL_SAFE, [0.8, 0.8, 0.8], 0.0), material(abi.MAT_COOK_TORR, [0.5, 0.4, 0.3], 0.2),
            material(abi.MAT_OREN_NAYAR, [0.2, 0.2, 0.2], 0.0)]
    ctx = FakeCtx(base)
    albedo = torch.tensor([[0.1, 0.1, 0.1], [0.25, 0.5, 0.75], [0.3, 0.3, 0.3]], requires_grad=True)
    rough = torch.tensor([0.9, 0.6, 0.1], requires_grad=True)
    img = AG.render(ctx, params(4, 3), albedo, rough, base=base)
    assert img.shape == (3, 4, 3)
    assert torch.all(img[..., 0] == 0.25)
    # the fail-safe entry keeps its own values; the others take the tensors'
    assert list(ctx.set[0].albedo) == pytest.approx([0.8, 0.8, 0.8]) and ctx.set[0].roughness == 0.0
    assert list(ctx.set[1].albedo) == pytest.approx([0.25, 0.5, 0.75]) and ctx.set[1].roughness == pytest.approx(0.6)
    assert ctx.set[2].roughness == pytest.approx(0.1)
    (img * torch.arange(3.0)).sum().backward()
    assert ctx.grad_in.shape == (3, 4, 3)
    np.testing.assert_array_equal(ctx.grad_in[0, 0], [0.0, 1.0, 2.0])
    np.testing.assert_array_equal(albedo.grad.numpy(), np.full((3, 3), 2.0))
    np.testing.assert_array_equal(rough.grad.numpy(), [0.0, 1.0, 2.0])


def test_stale_graph_and_bad_shapes_are_refused():
    base = [material(abi.MAT_OREN_NAYAR, [0.5, 0.5, 0.5], 0.0)] * 2
    ctx = FakeCtx(base)
    a = torch.full((2, 3), 0.5, requires_grad=True)
    r = torch.zeros(2, requires_grad=True)
    first = AG.render(ctx, params(2, 2), a, r, base=base)
    AG.render(ctx, params(2, 2), a, r, base=base)
    with pytest.raises(RuntimeError, match="another differentiable render"):
        first.sum().backward()
    with pytest.raises(ValueError):
        AG.render(ctx, params(2, 2), torch.zeros(3, 3), r, base=base)
    with pytest.raises(ValueError):
        AG.render(ctx, params(2, 2), a, torch.zeros(2, 1), base=base)


def test_image_and_gradients_follow_the_tensors_dtype():
    base = [material(abi.MAT_OREN_NAYAR, [0.5, 0.5, 0.5], 0.0), material(abi.MAT_COOK_TORR, [0.5, 0.4, 0.3], 0.2)]
    ctx = FakeCtx(base)
    a = torch.full((2, 3), 0.5, dtype=torch.float64, requires_grad=True)
    r = torch.full((2,), 0.3, dtype=torch.float32, requires_grad=True)
    img = AG.render(ctx, params(2, 2), a, r, base=base)
    assert img.dtype == torch.float64 and img.device == a.device
    img.sum().backward()
    assert a.grad.dtype == torch.float64 and r.grad.dtype == torch.float32
    np.testing.assert_array_equal(a.grad.numpy(), np.full((2, 3), 2.0))
