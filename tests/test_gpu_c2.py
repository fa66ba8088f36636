"""Parity on the benchmark configuration itself: the displaced icosphere of level 8 (1,310,730
triangles, 512 materials, 4 area lights) seen by the 1920x1080 camera, max depth 8, Russian
roulette from depth 3 at p = 0.5.

(b) Per-path radiance for 4,096 pixels on a uniform 64 x 64 grid over the whole frame (sky,
ground, sphere and silhouettes alike), in the product estimator (E8G_MODE_MIS) and the reference's
direct-lighting estimator (E8G_MODE_REF_LT1, unidirect_lt1 of pathtracer.cpp:587-653 with the
depth policy), with the reference's minstd streams and with Philox, on both fast trees and with the
integrators the benchmark times, against the oracle fed the same draws. The oracle's restatement
is pinned to the compiled reference bit for bit (test_oracle_pin.py).

(c) Converged images: the oracle renders three 64 x 64 crops of the frame (on the sphere, on the
ground, and across the sphere's silhouette and the ground's far edge) at 4,096 spp; the GPU renders
the whole frame at 4,096 spp with independent streams. The crops must agree within relMSE 1e-3
(mean over pixels and channels of (I - R)^2 / (R^2 + 1e-2)), for the reference's estimator against
itself, the product estimator against itself, and the product estimator against the reference's
estimator (both are unbiased for the same depth-capped integral).
"""
import os

import numpy as np
import pytest

import oracle_bind as ob
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.core import default_params

pytestmark = pytest.mark.gpu

W, H = 1920, 1080
POLICY = dict(max_depth=8, rr_start=3, rr_prob=0.5)
OPOL = ob.OPolicy(8, 3, 0.5, 8)
RTOL = 1e-4
CROPS = {"sphere": (928, 380), "ground": (1500, 900), "silhouette": (560, 480)}
CROP = 64


def match(a, b):
    ok = np.abs(a - b) <= np.maximum(RTOL * np.abs(b), 1e-6)
    return np.all(ok, axis=1)


def relmse(img, ref):
    img = img[..., :3].astype(np.float64)
    ref = ref[..., :3].astype(np.float64)
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


@pytest.fixture(scope="module")
def c2():
    sc = S.displaced_icosphere(level=8, seed=1, num_materials=512, width=W, height=H)
    return sc, ob.OracleScene(sc)


def grid_pixels():
    xs = np.linspace(0, W - 1, 64).round().astype(np.uint32)
    ys = np.linspace(0, H - 1, 64).round().astype(np.uint32)
    return (ys[:, None] * W + xs[None, :]).reshape(-1)


CASES = [(abi.BVH_SAH, abi.INTEGRATOR_MEGAKERNEL), (abi.BVH_WIDE, abi.INTEGRATOR_WAVEFRONT),
         (abi.BVH_WIDE, abi.INTEGRATOR_PLAIN)]


@pytest.mark.parametrize("layout,integ", CASES)
def test_c2_per_path_radiance_matches_oracle(ctx, c2, layout, integ):
    sc, osc = c2
    ctx.upload(sc, layout=layout)
    px = grid_pixels()
    samples = (np.arange(len(px)) % 64).astype(np.uint32)
    seed = 2024
    lines = []
    for mode in (abi.MODE_MIS, abi.MODE_REF_LT1):
        for rng in (abi.RNG_MINSTD, abi.RNG_PHILOX):
            p = default_params(mode, W, H, 1, seed=seed, rng=rng, **POLICY)
            # the wavefront integrator runs the MIS estimator; the reference's estimator runs on
            # the megakernel of the same tree
            p.integrator = integ if (mode == abi.MODE_MIS or integ != abi.INTEGRATOR_WAVEFRONT) \
                else abi.INTEGRATOR_MEGAKERNEL
            got = ctx.render_paths(p, px, samples)
            if rng == abi.RNG_MINSTD:
                seeds = np.array([ob.oracle().o_path_seed(seed, int(a), int(b)) for a, b in zip(px, samples)],
                                 np.uint32)
                ref = osc.render_paths(mode, W, H, px, seeds, policy=OPOL, threads=os.cpu_count() or 8)
            else:
                ref = osc.render_paths(mode, W, H, px, samples, policy=OPOL, rng=abi.RNG_PHILOX, seed=seed,
                                       threads=os.cpu_count() or 8)
            ok = match(got, ref)
            lines.append((mode, rng, float(ok.mean()), int((~ok).sum())))
    print("C2 per-path (layout %d, integrator %d): " % (layout, integ) +
          "; ".join("mode %d rng %d: %.5f (%d off)" % x for x in lines))
    for mode, rng, frac, _ in lines:
        assert frac >= 0.999, (mode, rng, frac)


def test_c2_converged_crops_match_oracle(ctx, c2):
    sc, osc = c2
    spp = 4096
    threads = os.cpu_count() or 8
    oracle_crops = {}
    for mode in (abi.MODE_REF_LT1, abi.MODE_MIS):
        for name, (x0, y0) in CROPS.items():
            oracle_crops[(mode, name)] = osc.render(mode, W, H, spp, seed=1, policy=OPOL, rng=abi.RNG_PHILOX,
                                                    crop=(x0, y0, x0 + CROP, y0 + CROP), threads=threads)
    gpu = {}
    ctx.upload(sc, layout=abi.BVH_WIDE)
    p = default_params(abi.MODE_MIS, W, H, spp, seed=4242, rng=abi.RNG_PHILOX, **POLICY)
    p.integrator = abi.INTEGRATOR_WAVEFRONT
    gpu[abi.MODE_MIS] = ctx.render(p)
    ctx.upload(sc, layout=abi.BVH_SAH)
    p = default_params(abi.MODE_REF_LT1, W, H, spp, seed=4242, rng=abi.RNG_PHILOX, **POLICY)
    gpu[abi.MODE_REF_LT1] = ctx.render(p)
    results = {}
    for name, (x0, y0) in CROPS.items():
        def crop(img):
            return img[y0:y0 + CROP, x0:x0 + CROP]
        results[("lt1/lt1", name)] = relmse(crop(gpu[abi.MODE_REF_LT1]), oracle_crops[(abi.MODE_REF_LT1, name)])
        results[("mis/mis", name)] = relmse(crop(gpu[abi.MODE_MIS]), oracle_crops[(abi.MODE_MIS, name)])
        results[("mis/lt1", name)] = relmse(crop(gpu[abi.MODE_MIS]), oracle_crops[(abi.MODE_REF_LT1, name)])
    print("C2 4096-spp crops, relMSE GPU vs oracle: " +
          "; ".join("%s %s %.2e" % (k[0], k[1], v) for k, v in results.items()))
    for k, v in results.items():
        assert v <= 1e-3, (k, v)
