"""Image rendering on the GPU: the image is the mean of the same per-path estimates the oracle
computes (identical draw streams), the furnace expectation of the reference's own test, and
basic invariants of pt_image_renderer::render."""
import numpy as np
import pytest

import golden_util as G
import oracle_bind as ob
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.core import default_params

pytestmark = pytest.mark.gpu


def rel_mse(img, ref, eps=1e-2):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + eps)))


@pytest.mark.parametrize("layout", [abi.BVH_REFERENCE, abi.BVH_SAH, abi.BVH_WIDE])
@pytest.mark.parametrize("mode", [abi.MODE_REF_LT1, abi.MODE_REF_UNI, abi.MODE_MIS, abi.MODE_REF_DIRECT,
                                  abi.MODE_REF_BDPT, abi.MODE_BDPT_POWER, abi.MODE_REF_LT2])
def test_image_matches_oracle_same_streams(ctx, mode, layout):
    """Same draw streams: >= 99.5% of pixels (8 paths each) agree to 1e-4; the rest are pixels
    with a path that took another branch after a last-ulp difference (sinf/cosf/atanf) or an edge
    tie."""
    sc = S.cornell(48, 40)
    ctx.upload(sc, layout=layout)
    osc = ob.OracleScene(sc)
    p = default_params(mode, 48, 40, 8, seed=9, max_depth=6 if mode == abi.MODE_MIS else 0)
    img = ctx.render(p)[..., :3]
    pol = ob.OPolicy(p.max_depth, p.rr_start, p.rr_prob, 8)  # e8g_default_params' policy for the mode
    ref = osc.render(mode, 48, 40, 8, seed=9, policy=pol, rng=p.rng)[..., :3]
    assert np.all(np.isfinite(img)) and np.all(img >= 0)
    close = np.all(np.abs(img - ref) <= np.maximum(1e-4 * np.abs(ref), 1e-6), axis=-1)
    assert close.mean() >= 0.995, close.mean()
    assert rel_mse(img, ref) < 2e-3, rel_mse(img, ref)


@pytest.mark.parametrize("mode", [abi.MODE_REF_UNI, abi.MODE_REF_LT1, abi.MODE_MIS, abi.MODE_REF_BDPT,
                                  abi.MODE_BDPT_POWER])
def test_furnace(ctx, mode):
    """tst_pathtracer.cpp:58-86 on the GPU: E[sum RGB] = 1 / (1 - 0.7) * 3 = 10 within 0.3."""
    ctx.upload(S.furnace(30))
    p = default_params(mode, 16, 16, 256, seed=13)
    img = ctx.render(p)
    mu = img[..., :3].sum(axis=-1).mean()
    assert abs(mu - 10.0) < 0.3, mu


def test_cornell_sanity_like_tst_renderer(ctx):
    """tst_renderer.cpp:117-168: no NaN/inf/negative pixels and enough total radiance."""
    ctx.upload(S.cornell(200, 150))
    p = default_params(abi.MODE_REF_LT1, 200, 150, 4)
    img = ctx.render(p)
    assert np.all(np.isfinite(img)) and np.all(img >= 0)
    assert np.all(img[..., :3].sum(axis=(0, 1)) > 1000)


def test_progressive_samples_add_up(ctx):
    ctx.upload(S.cornell(32, 32))
    full = ctx.render(default_params(abi.MODE_MIS, 32, 32, 8, seed=4))
    a = ctx.render(default_params(abi.MODE_MIS, 32, 32, 4, seed=4, sample_offset=0))
    b = ctx.render(default_params(abi.MODE_MIS, 32, 32, 4, seed=4, sample_offset=4))
    assert np.allclose(full, 0.5 * (a + b), rtol=1e-4, atol=1e-5)


def test_normal_and_position_tracers(ctx):
    d = G.load("cornell.npz")
    sc = G.scene_from(d)
    ctx.upload(sc)
    osc = ob.OracleScene(sc)
    for mode in (abi.MODE_NORMAL, abi.MODE_POSITION):
        img = ctx.render(default_params(mode, 64, 48, 1))
        ref = osc.render(mode, 64, 48, 1)
        assert np.allclose(img, ref, atol=1e-6)


def test_invalid_params(ctx):
    from x3dcore2_gb300.abi import E8GError
    ctx.upload(S.cornell(8, 8))
    for bad in (dict(width=1), dict(mode=42), dict(rr_prob=0.0), dict(rng=7), dict(max_depth=300),
                dict(rr_prob=1.0), dict(rr_start=100)):
        p = default_params(abi.MODE_REF_LT1, 8, 8, 1)
        for k, v in bad.items():
            setattr(p, k, v)
        with pytest.raises(E8GError, match="INVALID_ARG"):
            ctx.render(p)


def test_zero_spp_renders_black(ctx):
    ctx.upload(S.cornell(8, 8))
    img = ctx.render(default_params(abi.MODE_REF_LT1, 8, 8, 0))
    assert np.all(img[..., :3] == 0)


@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_WIDE])
@pytest.mark.parametrize("mode", [abi.MODE_MIS, abi.MODE_REF_LT1, abi.MODE_REF_UNI])
def test_plain_image_equals_megakernel(ctx, mode, layout):
    """The baseline one-thread-per-path kernel and the persistent megakernel run the same paths
    on the same streams: equal images up to the order of float accumulation."""
    sc = S.displaced_icosphere(level=5, seed=3, num_materials=32, width=96, height=54)
    ctx.upload(sc, layout=layout)
    p = default_params(mode, 96, 54, 8, seed=4, max_depth=8 if mode == abi.MODE_MIS else 0, rr_start=3)
    mk = ctx.render(p)
    p.integrator = abi.INTEGRATOR_PLAIN
    pl = ctx.render(p)
    close = np.abs(pl - mk) <= np.maximum(1e-4 * np.abs(mk), 1e-5)
    assert close.mean() >= 0.999, close.mean()


def test_converged_mis_agrees_with_reference_estimator(ctx):
    """Check (c) on the Cornell box of the first benchmark configuration at 256x256: the product
    estimator (NEE + BSDF sampling, power heuristic) and the reference's unidirect_lt1 estimator,
    both at 4096 spp with independent streams and the reference's unbounded Russian-roulette
    policy, agree within relMSE 1e-3 (epsilon 1e-2 in the denominator)."""
    ctx.upload(S.cornell(256, 256))
    a = ctx.render(default_params(abi.MODE_MIS, 256, 256, 4096, seed=21))[..., :3]
    b = ctx.render(default_params(abi.MODE_REF_LT1, 256, 256, 4096, seed=22))[..., :3]
    assert rel_mse(a, b) < 1e-3, rel_mse(a, b)


@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_WIDE])
@pytest.mark.parametrize("capacity_small", [False, True])
def test_wavefront_image_equals_megakernel(ctx, capacity_small, layout):
    """Same estimator, same streams: the wavefront image equals the megakernel image up to the
    order of float accumulation; with few slots the queues refill many times."""
    import ctypes as C
    sc = S.displaced_icosphere(level=5, seed=3, num_materials=32, width=96, height=54)
    ctx.upload(sc, layout=layout)
    p = default_params(abi.MODE_MIS, 96, 54, 16, seed=2, max_depth=8, rr_start=3)
    mk = ctx.render(p)
    if capacity_small:
        # tune on this frame, then force refills with the smallest candidate by rendering more spp
        r = abi.TuneResult()
        abi.check(ctx.lib.e8g_wavefront_tune(ctx.h, C.byref(p), C.byref(r)), ctx.h, "tune")
        assert r.num_candidates == 50 and r.capacity in tuple(1 << k for k in range(20, 25))
        assert r.threshold in (4, 8, 12, 16, 24) and r.bounces_per_graph in (2, 4)
        assert all(ms > 0 for ms in r.cand_ms[:50])
    p.integrator = abi.INTEGRATOR_WAVEFRONT
    wf = ctx.render(p)
    assert np.all(np.isfinite(wf)) and np.all(wf >= 0)
    close = np.abs(wf - mk) <= np.maximum(1e-4 * np.abs(mk), 1e-5)
    assert close.mean() >= 0.999, close.mean()


def test_bdpt_power_converges_to_mis(ctx):
    """Two unbiased estimators of the same truncated integral (paths of at most 6 surface
    vertices): power-heuristic BDPT with subpaths capped at 3 and MIS with depth 5 agree on the
    Cornell box at 1024 spp to within 1% of the frame mean."""
    ctx.upload(S.cornell(64, 64))
    a = ctx.render(default_params(abi.MODE_BDPT_POWER, 64, 64, 1024, seed=2, bdpt_max_len=3))[..., :3]
    b = ctx.render(default_params(abi.MODE_MIS, 64, 64, 1024, seed=3, max_depth=5, rr_start=100, rr_prob=0.5))[..., :3]
    assert abs(a.mean() - b.mean()) <= 0.01 * b.mean(), (a.mean(), b.mean())
    assert rel_mse(a, b) < 5e-3


@pytest.mark.parametrize("mode,rng", [(abi.MODE_REF_UNI, abi.RNG_MINSTD), (abi.MODE_REF_LT1, abi.RNG_MINSTD),
                                      (abi.MODE_MIS, abi.RNG_PHILOX)])
def test_firefly_clamp_matches_oracle(ctx, mode, rng):
    """firefly = 1 (renderer.cpp:46-83): every sample image is clamped against its neighbours
    before it is accumulated. The oracle renders the same paths (same streams), applies its
    restatement of the clamp per sample and averages; the GPU image equals it on >= 98% of
    pixels, and the clamp changes the image."""
    sc = S.cornell(40, 32)
    ctx.upload(sc)
    w, h, spp = 40, 32, 6
    p = default_params(mode, w, h, spp, seed=5, rng=rng, firefly=1)
    got = ctx.render(p)[..., :3]
    p.firefly = 0
    plain = ctx.render(p)[..., :3]
    osc = ob.OracleScene(sc)
    pol = ob.REF_POLICY  # e8g_default_params: the reference's policy for every mode
    px = np.arange(w * h, dtype=np.uint32)
    acc = np.zeros((h, w, 3), np.float32)
    for s in range(spp):
        if rng == abi.RNG_MINSTD:
            seeds = np.array([ob.oracle().o_path_seed(5, int(q), s) for q in px], np.uint32)
            est = osc.render_paths(mode, w, h, px, seeds, policy=pol)
        else:
            est = osc.render_paths(mode, w, h, px, np.full(w * h, s, np.uint32), policy=pol, rng=rng, seed=5)
        ob.firefly_add(est.reshape(h, w, 3), acc)
    ref = acc * np.float32(1.0 / spp)
    close = np.all(np.abs(got - ref) <= np.maximum(1e-4 * np.abs(ref), 1e-6), axis=-1)
    assert close.mean() >= 0.995, close.mean()
    assert not np.allclose(got, plain)


def test_lt2_furnace_equals_oracle(ctx):
    """bidirect_lt2 in the furnace of tst_pathtracer.cpp: the reference's estimator is not
    unbiased there (its mean is about 9.2, not 10: the oracle reproduces the reference bit for
    bit). The GPU render equals the oracle's mean for the same streams."""
    ctx.upload(S.furnace(30))
    w = h = 16
    spp = 128
    img = ctx.render(default_params(abi.MODE_REF_LT2, w, h, spp, seed=13))
    osc = ob.OracleScene(S.furnace(30))
    ref = osc.render(abi.MODE_REF_LT2, w, h, spp, seed=13)
    g, o = float(img[..., :3].sum(axis=-1).mean()), float(ref[..., :3].sum(axis=-1).mean())
    assert abs(g - o) <= 1e-3 * o, (g, o)
    assert 8.5 < o < 9.6


def test_progressive_accumulation_equals_one_render(ctx):
    """e8g_render_progressive: four calls of 4 spp continue the sample sequence in the device
    accumulator and give the image of one 16-spp render; reset starts over; a plain render in
    between ends the sequence."""
    import torch
    ctx.upload(S.cornell(64, 48))
    p = default_params(abi.MODE_MIS, 64, 48, 4, seed=7)
    d = torch.empty((48, 64, 4), dtype=torch.float32, device="cuda")
    for k in range(4):
        ctx.render_progressive(p, d.data_ptr(), reset=(k == 0))
    torch.cuda.synchronize()
    prog = d.cpu().numpy()
    one = ctx.render(default_params(abi.MODE_MIS, 64, 48, 16, seed=7))
    close = np.abs(prog - one) <= np.maximum(1e-5 * np.abs(one), 1e-6)
    assert close.mean() >= 0.999, close.mean()
    # after a plain render the next progressive call starts a new sequence at sample 0
    ctx.render_progressive(p, d.data_ptr())
    torch.cuda.synchronize()
    first = d.cpu().numpy()
    four = ctx.render(p)
    assert np.allclose(first, four, rtol=1e-5, atol=1e-6)


def test_wavefront_set_pins_the_configuration(ctx):
    """e8g_wavefront_set: any valid configuration renders the same image (the paths are the
    same; only slot counts and graph sizes change); out-of-range values are refused."""
    sc = S.displaced_icosphere(level=4, seed=2, num_materials=8, width=64, height=48)
    ctx.upload(sc, layout=abi.BVH_WIDE)
    p = default_params(abi.MODE_MIS, 64, 48, 8, seed=6, max_depth=8, rr_start=3,
                       integrator=abi.INTEGRATOR_WAVEFRONT)
    imgs = []
    for cap, b, th in ((1 << 12, 1, 0), (1 << 16, 8, 24), (1 << 20, 2, 12)):
        abi.check(ctx.lib.e8g_wavefront_set(ctx.h, cap, b, th), ctx.h, "set")
        imgs.append(ctx.render(p))
    for im in imgs[1:]:
        close = np.abs(im - imgs[0]) <= np.maximum(1e-4 * np.abs(imgs[0]), 1e-5)
        assert close.mean() >= 0.999
    for bad in ((512, 2, 12), (1 << 20, 0, 12), (1 << 20, 2, 33)):
        assert ctx.lib.e8g_wavefront_set(ctx.h, *bad) == 1  # E8G_ERR_INVALID_ARG


@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_WIDE])
@pytest.mark.parametrize("mode", [abi.MODE_REF_LT1, abi.MODE_MIS, abi.MODE_REF_BDPT, abi.MODE_BDPT_POWER])
def test_mixture_and_fail_safe_image_matches_oracle(ctx, mode, layout):
    """The mixture fixture's room (a wall without a material, mixtures of a Lambert wall with a
    GGX metal and of that metal with a rough Oren-Nayar, material.cpp:54-106) rendered as a whole
    image on the fast trees: equal to the oracle's image of the same streams (the oracle equals
    the compiled reference on this scene path for path)."""
    d = G.load("mixture.npz")
    sc = G.scene_from(d)
    w, h = int(d["width"]), int(d["height"])
    ctx.upload(sc, layout=layout)
    osc = ob.OracleScene(sc)
    p = default_params(mode, w, h, 4, seed=21, max_depth=6 if mode == abi.MODE_MIS else 0, bdpt_max_len=6)
    img = ctx.render(p)[..., :3]
    pol = ob.OPolicy(p.max_depth, p.rr_start, p.rr_prob, p.bdpt_max_len)
    ref = osc.render(mode, w, h, 4, seed=21, policy=pol, rng=p.rng)[..., :3]
    assert np.all(np.isfinite(img)) and np.all(img >= 0) and img.sum() > 0
    close = np.all(np.abs(img - ref) <= np.maximum(1e-4 * np.abs(ref), 1e-6), axis=-1)
    print(f"mixture image mode {mode} layout {layout}: {close.mean():.5f} of pixels within 1e-4")
    assert close.mean() >= 0.995, close.mean()


def test_wavefront_kernel_timing_leaves_the_image_and_fills_the_stats(ctx):
    """e8g_set_kernel_timing: event records in the bounce graph time the trace and shading kernels;
    the image is the untimed one (identical paths), the kernel times fit inside the render's."""
    import ctypes as C
    sc = S.cornell(96, 64)
    ctx.upload(sc, layout=abi.BVH_WIDE)
    p = default_params(abi.MODE_MIS, 96, 64, 8, seed=3, max_depth=6, integrator=abi.INTEGRATOR_WAVEFRONT)
    plain = ctx.render(p)
    assert ctx.stats()["trace_ms"] == 0.0
    ctx.set_kernel_timing(True)
    try:
        timed = ctx.render(p)
        st = ctx.stats()
    finally:
        ctx.set_kernel_timing(False)
    close = np.all(np.abs(timed - plain) <= np.maximum(1e-4 * np.abs(plain), 1e-6), axis=-1)
    assert close.mean() >= 0.999
    assert st["trace_ms"] > 0 and st["shade_ms"] > 0 and st["trace_launches"] > 0
    assert st["trace_ms"] + st["shade_ms"] <= st["kernel_ms"] * 1.001
    gbs = C.c_double()
    assert ctx.lib.e8g_l2_read_bandwidth(ctx.h, 64 << 20, 4, C.byref(gbs)) == 0
    assert 1000 < gbs.value < 100000, gbs.value  # GB/s: far above HBM's few TB/s, below nonsense


def test_wavefront_tuner_cache_and_shade_shapes(ctx, tmp_path):
    """e8g_wavefront_tune searches the shading kernel's block shapes too; e8g_wavefront_tune_cached
    writes its choice to a JSON file keyed by the scene and frame size bucket and takes it from
    there the next time; every shape renders the same image."""
    import ctypes as C
    import json
    sc = S.cornell(128, 96)
    ctx.upload(sc, layout=abi.BVH_WIDE)
    p = default_params(abi.MODE_MIS, 128, 96, 4, seed=3, max_depth=6, integrator=abi.INTEGRATOR_WAVEFRONT)
    path = str(tmp_path / "tune.json").encode()
    r = abi.TuneResult()
    assert ctx.lib.e8g_wavefront_tune_cached(ctx.h, C.byref(p), path, C.byref(r)) == 0
    assert r.from_cache == 0 and r.num_shade == 8 and r.shade_variant < 8
    assert all(r.shade_ms[i] > 0 for i in range(8))
    with open(path) as f:
        d = json.load(f)
    (key, entry), = d.items()
    assert "layout2" in key and entry["capacity"] == r.capacity and entry["shade"] == r.shade_variant
    assert entry["concurrent"] == r.concurrent and r.concurrent_ms[0] > 0 and r.concurrent_ms[1] > 0
    r2 = abi.TuneResult()
    assert ctx.lib.e8g_wavefront_tune_cached(ctx.h, C.byref(p), path, C.byref(r2)) == 0
    assert r2.from_cache == 1 and (r2.capacity, r2.bounces_per_graph, r2.threshold, r2.shade_variant) == \
        (r.capacity, r.bounces_per_graph, r.threshold, r.shade_variant)
    base = None
    for v in range(8):
        assert ctx.lib.e8g_wavefront_set_shade(ctx.h, v) == 0
        img = ctx.render(p)
        if base is None:
            base = img
        close = np.all(np.abs(img - base) <= np.maximum(1e-4 * np.abs(base), 1e-6), axis=-1)
        assert close.mean() >= 0.999, v
    assert ctx.lib.e8g_wavefront_set_shade(ctx.h, 8) == 1


@pytest.mark.parametrize("layout", [abi.BVH_WIDE, abi.BVH_SAH])
def test_bdpt_power_split_form_renders_the_same_image(ctx, layout):
    """The split form of power-heuristic BDPT (E8G_INTEGRATOR_WAVEFRONT: subpath kernel,
    connection kernel and the wavefront's shadow-ray trace per chunk of paths) renders the same
    paths as one thread per path: the same image (the terms of a path added in another order),
    also when a memory limit forces chunks of a few thousand paths; its counted run is the
    one-thread form's (the same rays)."""
    d = G.load("ico.npz")
    sc = G.scene_from(d)
    ctx.upload(sc, layout=layout)
    w, h = int(d["width"]), int(d["height"])
    p = default_params(abi.MODE_BDPT_POWER, w, h, 8, seed=4, bdpt_max_len=6)
    one = ctx.render(p)
    c1 = ctx.count_traversal(p)
    p.integrator = abi.INTEGRATOR_WAVEFRONT
    ctx.set_memory_limit(ctx.memory_used() + 12 * 1024 * 1024)  # chunks of about 4,000 paths
    try:
        chunked = ctx.render(p)
    finally:
        ctx.set_memory_limit(0)
    c2 = ctx.count_traversal(p)
    split = ctx.render(p)  # one chunk
    for img, name in ((chunked, "chunked"), (split, "one chunk")):
        close = np.all(np.abs(img - one) <= np.maximum(1e-4 * np.abs(one), 1e-6), axis=-1)
        print(f"split bdpt layout {layout} {name}: {close.mean():.5f} of pixels within 1e-4")
        assert close.mean() >= 0.999, (name, close.mean())
    assert (c1["rays"], c1["nodes"], c1["tris"]) == (c2["rays"], c2["nodes"], c2["tris"])


@pytest.mark.parametrize("mode", [abi.MODE_REF_BDPT, abi.MODE_BDPT_POWER])
def test_bidirectional_traversal_counts(ctx, mode):
    """e8g_count_traversal covers the bidirectional kernels (the roofline's algorithmic bytes): the
    counted render traces rays, fetches node boxes and tests triangles, and its image is the
    uncounted one."""
    sc = S.cornell(64, 48)
    ctx.upload(sc, layout=abi.BVH_WIDE)
    p = default_params(mode, 64, 48, 4, seed=2, bdpt_max_len=6)
    img = ctx.render(p)
    c = ctx.count_traversal(p)
    assert c["counted"] == 1 and c["rays"] > 64 * 48 * 4 and c["nodes"] > c["rays"] and c["tris"] > 0
    again = ctx.render(p)
    np.testing.assert_allclose(again, img, rtol=1e-5, atol=1e-6)
    with pytest.raises(Exception, match="UNSUPPORTED"):
        ctx.count_traversal(default_params(abi.MODE_REF_LT2, 64, 48, 1))


@pytest.mark.parametrize("layout", [abi.BVH_WIDE, abi.BVH_SAH])
def test_concurrent_wavefront_renders_the_same_paths(ctx, layout):
    """e8g_wavefront_set_concurrent: two slot pools interleaving on two streams render the same
    paths as one pool: the image equals the megakernel's, and per-path radiance equals the
    oracle's, for a frame much larger than the slot pools (slots refill many times)."""
    import ctypes as C
    sc = S.displaced_icosphere(level=4, seed=3, num_materials=16, width=160, height=120)
    ctx.upload(sc, layout=layout)
    p = default_params(abi.MODE_MIS, 160, 120, 16, seed=7, max_depth=8, rr_start=3)
    ref = ctx.render(p)
    assert ctx.lib.e8g_wavefront_set(ctx.h, 4096, 2, 12 if layout == abi.BVH_WIDE else 16) == 0
    assert ctx.lib.e8g_wavefront_set_concurrent(ctx.h, 1) == 0
    try:
        p.integrator = abi.INTEGRATOR_WAVEFRONT
        img = ctx.render(p)
        close = np.all(np.abs(img - ref) <= np.maximum(1e-4 * np.abs(ref), 1e-6), axis=-1)
        assert close.mean() >= 0.999, close.mean()
        px = np.random.default_rng(4).integers(0, 160 * 120, 2000).astype(np.uint32)
        smp = np.arange(len(px), dtype=np.uint32)
        got = ctx.render_paths(p, px, smp)
        osc = ob.OracleScene(sc)
        want = osc.render_paths(abi.MODE_MIS, 160, 120, px, smp, policy=ob.OPolicy(8, 3, 0.5, 8),
                                rng=abi.RNG_PHILOX, seed=7)
        ok = np.all(np.abs(got - want) <= np.maximum(1e-4 * np.abs(want), 1e-6), axis=1)
        assert ok.mean() >= 0.999, ok.mean()
    finally:
        ctx.lib.e8g_wavefront_set_concurrent(ctx.h, 0)
        ctx.lib.e8g_wavefront_set(ctx.h, 1 << 21, 4, 16)
