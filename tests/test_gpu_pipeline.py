"""The render pipeline's frame (e8g_pipeline_frame) on the GPU: a frame is the render of the
configured tracer followed by the ACES compositor, as pt_render_pipeline::render_frame composes
them (pipeline.cpp:73-101); changes between frames are committed; progressive frames accumulate
to the image of one longer render."""
import numpy as np
import pytest

from test_gpu_update import same_image
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.core import default_params, pipeline_config

pytestmark = pytest.mark.gpu


def test_frame_is_render_then_aces(ctx):
    sc = S.cornell(64, 48)
    ctx.upload(sc, build=False)
    cfg = pipeline_config(path_tracer="unidirectional_lt1", samples_per_frame=8, auto_exposure=True)
    px, rgba = ctx.pipeline_frame(cfg, 64, 48, want_rgba=True)
    p = default_params(abi.MODE_REF_LT1, 64, 48, 8)
    want = ctx.render(p)
    assert same_image(rgba, want)
    # the pixels are the compositor's on that very float frame
    assert np.array_equal(px, ctx.composite(rgba, abi.TONEMAP_ACES, True, 1.0))
    # the reference re-renders the same frame every time
    px2, _ = ctx.pipeline_frame(cfg, 64, 48)
    assert np.abs(px2.astype(int) - px.astype(int)).max() <= 1


def test_progressive_frames_accumulate(ctx):
    sc = S.cornell(64, 48)
    ctx.upload(sc)
    cfg = pipeline_config(path_tracer="mis", samples_per_frame=4, progressive=True, exposure=1.3)
    for _ in range(4):
        _, rgba = ctx.pipeline_frame(cfg, 64, 48, want_rgba=True)
    one = ctx.render(default_params(abi.MODE_MIS, 64, 48, 16))
    assert same_image(rgba, one)


def test_scene_change_between_frames_is_committed(ctx):
    sc = S.cornell(48, 48)
    ctx.upload(sc)
    cfg = pipeline_config(path_tracer="mis", samples_per_frame=4, progressive=True)
    _, a = ctx.pipeline_frame(cfg, 48, 48, want_rgba=True)
    lm = sc.lights[0].mesh
    v0, v1 = sc.voff[lm], sc.voff[lm + 1]
    m = np.eye(4, dtype=np.float32)
    m[1, 3] = -0.05  # the light moves down
    ctx.transform_mesh(lm, m)
    _, b = ctx.pipeline_frame(cfg, 48, 48, want_rgba=True)  # commits, restarts the accumulation
    one = ctx.render(default_params(abi.MODE_MIS, 48, 48, 4))
    assert same_image(b, one) and not same_image(a, b)
    assert v1 > v0


def test_firefly_and_progressive_refused(ctx):
    ctx.upload(S.cornell(16, 16))
    cfg = pipeline_config(progressive=True, firefly_filter=True)
    with pytest.raises(abi.E8GError, match="UNSUPPORTED"):
        ctx.pipeline_frame(cfg, 16, 16)
