"""e8g_render_dev_noalloc: the render entry point that allocates no device memory.

It is for callers that cannot call cudaMalloc while rendering (cudaMalloc synchronises the device
and fails once a process has committed all of its device memory up front). Its scratch lives in
a fixed-size device array owned by the library; this test checks, through the C ABI, that two
calls in a row give the same image as the allocating entry point e8g_render_dev (to the 1e-4
tolerance of the other image tests: only the order of the float accumulation differs) for the
three integrators and the SAH and eight-wide trees, at the largest image it takes (exactly
E8G_NOALLOC_MAX_PIXELS pixels), that the device's free memory is the same before and after a
call, and that images above the array's capacity are refused. Kept in its own file, collected
last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, ctx, p, out, stream):
    from x3dcore2_gb300 import abi
    st = lib.e8g_render_dev_noalloc(ctx.h, C.byref(p), C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert st == abi.E8G_OK, lib.e8g_last_error(ctx.h)


def _close(a, b):
    return np.all(np.abs(a - b) <= np.maximum(1e-4 * np.abs(b), 1e-6))


def test_noalloc_matches_render_dev_on_two_calls_in_a_row(lib):
    import torch

    from x3dcore2_gb300 import abi
    from x3dcore2_gb300 import scene as S
    from x3dcore2_gb300.core import Context, default_params

    w, h = 128, 96
    with Context(0) as ctx:
        ctx.upload(S.cornell(w, h))
        stream = torch.cuda.current_stream()
        ref = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
        out = torch.empty_like(ref)
        for mode in (abi.MODE_MIS, abi.MODE_REF_LT1, abi.MODE_REF_BDPT):
            p = default_params(mode, w, h, 4, seed=7, max_depth=8 if mode == abi.MODE_MIS else 0)
            ctx.render_dev(p, ref.data_ptr(), stream.cuda_stream)
            torch.cuda.synchronize()
            b = ref.cpu().numpy()
            for _ in range(2):
                out.fill_(-1.0)
                torch.cuda.synchronize()
                _noalloc(lib, ctx, p, out, stream)
                torch.cuda.synchronize()
                assert _close(out.cpu().numpy(), b), mode
        # beyond the fixed capacity: refused, nothing launched
        p = default_params(abi.MODE_MIS, 512, 512, 1)
        big = torch.empty((512, 512, 4), dtype=torch.float32, device="cuda")
        st = lib.e8g_render_dev_noalloc(ctx.h, C.byref(p), C.c_void_p(big.data_ptr()), None)
        assert st == 1 and b"E8G_NOALLOC_MAX_PIXELS" in lib.e8g_last_error(ctx.h)


def test_noalloc_at_capacity_every_integrator_and_tree_no_memory_taken(lib):
    import torch

    from x3dcore2_gb300 import abi
    from x3dcore2_gb300 import scene as S
    from x3dcore2_gb300.core import Context, default_params

    w = h = 256  # exactly E8G_NOALLOC_MAX_PIXELS
    assert w * h == 65536
    stream = torch.cuda.current_stream()
    ref = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    out = torch.empty_like(ref)
    with Context(0) as ctx:
        for layout in (abi.BVH_SAH, abi.BVH_WIDE):
            ctx.upload(S.cornell(w, h), layout=layout)
            for integ in (abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_PLAIN, abi.INTEGRATOR_WAVEFRONT):
                p = default_params(abi.MODE_MIS, w, h, 2, seed=11, max_depth=6, integrator=integ)
                ctx.render_dev(p, ref.data_ptr(), stream.cuda_stream)
                torch.cuda.synchronize()
                b = ref.cpu().numpy()
                _noalloc(lib, ctx, p, out, stream)  # first call on the device: address lookup
                torch.cuda.synchronize()
                for _ in range(2):
                    out.fill_(-1.0)
                    torch.cuda.synchronize()
                    free0, _ = torch.cuda.mem_get_info()
                    _noalloc(lib, ctx, p, out, stream)
                    torch.cuda.synchronize()
                    free1, _ = torch.cuda.mem_get_info()
                    assert free1 == free0, (layout, integ, free0 - free1)
                    assert _close(out.cpu().numpy(), b), (layout, integ)
        # one pixel row more than the capacity: refused
        p = default_params(abi.MODE_MIS, w, h + 1, 1)
        st = lib.e8g_render_dev_noalloc(ctx.h, C.byref(p), C.c_void_p(out.data_ptr()), None)
        assert st == 1 and b"E8G_NOALLOC_MAX_PIXELS" in lib.e8g_last_error(ctx.h)
