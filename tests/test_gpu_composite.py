"""e8g_composite / e8g_composite_dev: the reference's compositors on the device, against the
oracle's restatement (itself equal to the compiled reference, tests/test_oracle_pin.py). powf
and the exposure's log/exp sums differ from glibc's in their last bits, so a pixel on a rounding
edge may land one 8-bit step away; nothing further."""
import numpy as np
import pytest

import golden_util as G
import oracle_bind as ob
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.core import default_params

pytestmark = pytest.mark.gpu


def close_8bit(a, b, min_exact):
    diff = np.abs(a.astype(np.int32) - b.astype(np.int32))
    return diff.max() <= 1 and (diff == 0).mean() >= min_exact


@pytest.mark.parametrize("tonemap", [abi.TONEMAP_CLAMP, abi.TONEMAP_ACES])
@pytest.mark.parametrize("auto", [True, False])
def test_composite_matches_reference_golden(ctx, tonemap, auto):
    d = G.load("composite.npz")
    got = ctx.composite(d["image"], tonemap, auto, 0.8)
    name = ("clamp" if tonemap == abi.TONEMAP_CLAMP else "aces") + ("_auto" if auto else "_fixed")
    assert close_8bit(got, d[name], 0.99)


def test_composite_of_a_render(ctx):
    """A rendered frame through e8g_render_dev and e8g_composite_dev stays on the device; the
    8-bit image equals the oracle's compositing of the same float image."""
    import torch
    ctx.upload(S.cornell(96, 64))
    p = default_params(abi.MODE_MIS, 96, 64, 16, seed=3)
    d_img = torch.empty((64, 96, 4), dtype=torch.float32, device="cuda")
    d_px = torch.empty((64, 96, 4), dtype=torch.uint8, device="cuda")
    ctx.render_dev(p, d_img.data_ptr())
    torch.cuda.synchronize()
    cp = abi.CompositeParams(abi.TONEMAP_ACES, 1, 1.0)
    import ctypes as C
    abi.check(ctx.lib.e8g_composite_dev(ctx.h, C.c_void_p(d_img.data_ptr()), 96, 64, C.byref(cp),
                                        C.c_void_p(d_px.data_ptr()), None), ctx.h, "e8g_composite_dev")
    torch.cuda.synchronize()
    ref = ob.composite(d_img.cpu().numpy(), abi.TONEMAP_ACES, True)
    assert close_8bit(d_px.cpu().numpy(), ref, 0.97)


def test_composite_rejects_bad_arguments(ctx):
    from x3dcore2_gb300.abi import E8GError
    with pytest.raises(E8GError, match="INVALID_ARG"):
        ctx.composite(np.zeros((4, 4, 4), np.float32), tonemap=7)
