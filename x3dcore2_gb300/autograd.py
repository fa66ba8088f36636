"""torch.autograd binding of the path-replay adjoint (e8g_forward / e8g_backward).

`render(ctx, params, albedo, roughness)` renders the uploaded scene with per-material albedo
(num_materials, 3) and roughness (num_materials,) taken from the tensors, and returns the
(height, width, 3) image; its backward replays every path on the device and returns
dLoss/d(albedo) and dLoss/d(roughness). Only Oren-Nayar and Cook-Torrance materials take the
tensors' values (the fail-safe and mixture entries keep theirs and get zero gradients), as
e8g_backward defines. The tensors may live on any device and in any floating dtype: their values
cross the C ABI as host float32, the image comes back on albedo's device and dtype, and each
gradient on its own tensor's device and dtype.

e8g_backward replays the last e8g_forward of its context, so a graph's backward must run before
another differentiable render on the same context; the binding checks this and raises.
"""
import numpy as np
import torch

from . import abi


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(fctx, albedo, roughness, ctx, params, base):
        nm = len(base)
        a = albedo.detach().to(torch.float32).cpu().numpy().reshape(nm, 3)
        r = roughness.detach().to(torch.float32).cpu().numpy().reshape(nm)
        mats = []
        for k, m in enumerate(base):
            q = abi.Material.from_buffer_copy(m)
            if q.type in (abi.MAT_OREN_NAYAR, abi.MAT_COOK_TORR):
                q.albedo[:] = [float(x) for x in a[k]]
                q.roughness = float(r[k])
            mats.append(q)
        ctx.set_materials(mats)
        img = ctx.forward(params)
        ctx._adjoint_token = getattr(ctx, "_adjoint_token", 0) + 1
        fctx.core = ctx
        fctx.token = ctx._adjoint_token
        fctx.shape = (params.height, params.width)
        fctx.like = ((albedo.device, albedo.dtype), (roughness.device, roughness.dtype))
        out = torch.from_numpy(np.ascontiguousarray(img[..., :3]))
        return out.to(device=albedo.device, dtype=albedo.dtype)

    @staticmethod
    def backward(fctx, grad_img):
        ctx = fctx.core
        if getattr(ctx, "_adjoint_token", None) != fctx.token:
            raise RuntimeError("another differentiable render ran on this context since this one's forward")
        h, w = fctx.shape
        g = grad_img.detach().to(torch.float32).cpu().numpy().reshape(h, w, 3)
        da, dr = ctx.backward(g)
        (ad, at), (rd, rt) = fctx.like
        return (torch.from_numpy(da).to(device=ad, dtype=at), torch.from_numpy(dr).to(device=rd, dtype=rt),
                None, None, None)


def render(ctx, params, albedo, roughness, base=None):
    """Differentiable render: image (height, width, 3) as a function of albedo and roughness.
    `base` is the material table whose other fields are kept (default: the uploaded scene's);
    params must ask for E8G_MODE_MIS with Philox streams (the paths the adjoint replays)."""
    if base is None:
        base = ctx.scene.material_list()
    if albedo.shape != (len(base), 3) or roughness.shape != (len(base),):
        raise ValueError("albedo must be (num_materials, 3) and roughness (num_materials,)")
    return _Render.apply(albedo, roughness, ctx, params, base)
