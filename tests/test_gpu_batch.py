"""e8g_batch_render: independent scenes of different sizes, resolutions, sample counts and depth
policies in one persistent launch give the same images as rendering each scene alone."""
import numpy as np
import pytest

from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.core import default_params, render_batch

pytestmark = pytest.mark.gpu


def test_batch_equals_separate_renders(ctx):
    rng = np.random.default_rng(4)
    scenes, params = [], []
    for k in range(6):
        ntri = int(np.exp(rng.uniform(np.log(1000), np.log(40000))))
        w, h = [(32, 32), (48, 40), (64, 64), (40, 24)][k % 4]
        sc = S.soup(ntri, seed=k + 1, width=w, height=h, roughness_lo=0.02, roughness_hi=1.0)
        mode = [abi.MODE_MIS, abi.MODE_REF_LT1, abi.MODE_MIS][k % 3]
        p = default_params(mode, w, h, [4, 16, 8][k % 3], seed=k + 3,
                           max_depth=int(rng.integers(4, 11)) if mode == abi.MODE_MIS else 0, rr_start=3)
        scenes.append(sc)
        params.append(p)
    imgs, st = render_batch(ctx, scenes, params)
    assert st["launches"] == 3 and st["paths"] == sum(p.width * p.height * p.spp for p in params)
    for sc, p, img in zip(scenes, params, imgs):
        ctx.upload(sc)
        ref = ctx.render(p)
        close = np.abs(img - ref) <= np.maximum(1e-4 * np.abs(ref), 1e-5)
        assert close.mean() >= 0.999, close.mean()


def test_batch_rejects_bad_items(ctx):
    from x3dcore2_gb300.abi import E8GError
    sc = S.cornell(16, 16)
    p = default_params(abi.MODE_REF_BDPT, 16, 16, 1)
    with pytest.raises(E8GError, match="UNSUPPORTED"):
        render_batch(ctx, [sc], [p])
    p = default_params(abi.MODE_MIS, 16, 16, 1, firefly=1)
    with pytest.raises(E8GError, match="UNSUPPORTED"):
        render_batch(ctx, [sc], [p])


def test_batch_mixes_stream_kinds(ctx):
    """A batch whose scenes use different stream kinds (the reference's minstd, Philox) runs
    one launch; each scene's image equals its separate render."""
    scenes = [S.cornell(24, 24), S.cornell(24, 24)]
    params = [default_params(abi.MODE_REF_LT1, 24, 24, 4, seed=3, rng=abi.RNG_MINSTD),
              default_params(abi.MODE_REF_LT1, 24, 24, 4, seed=3, rng=abi.RNG_PHILOX)]
    imgs, st = render_batch(ctx, scenes, params)
    assert st["launches"] == 3
    assert not np.allclose(imgs[0], imgs[1])
    for sc, p, img in zip(scenes, params, imgs):
        ctx.upload(sc)
        ref = ctx.render(p)
        close = np.abs(img - ref) <= np.maximum(1e-4 * np.abs(ref), 1e-5)
        assert close.mean() >= 0.999, close.mean()


def test_batch_wavefront_equals_separate_renders(ctx):
    """The many-scene wavefront (eight-wide trees, slots shared by every scene, one graph-captured
    bounce loop): each scene's image equals its separate wavefront render on the same tree, for
    scenes of different sizes, resolutions, sample counts and depth policies."""
    rng = np.random.default_rng(8)
    scenes, params = [], []
    for k in range(7):
        ntri = int(np.exp(rng.uniform(np.log(1000), np.log(60000))))
        w, h = [(32, 32), (48, 40), (64, 64), (40, 24)][k % 4]
        sc = S.soup(ntri, seed=20 + k, width=w, height=h, roughness_lo=0.02, roughness_hi=1.0)
        p = default_params(abi.MODE_MIS, w, h, [4, 16, 8][k % 3], seed=k + 5, max_depth=int(rng.integers(4, 11)),
                           rr_start=3, integrator=abi.INTEGRATOR_WAVEFRONT)
        scenes.append(sc)
        params.append(p)
    imgs, st = render_batch(ctx, scenes, params)
    assert st["launches"] >= 5  # first hits, reset + shade + trace per bounce, resolve
    for sc, p, img in zip(scenes, params, imgs):
        ctx.upload(sc, layout=abi.BVH_WIDE)
        ref = ctx.render(p)
        close = np.abs(img - ref) <= np.maximum(1e-4 * np.abs(ref), 1e-5)
        assert close.mean() >= 0.999, close.mean()
