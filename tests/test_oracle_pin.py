"""Pins the oracle (C restatement) to the reference: golden fixtures made by the compiled reference,
and, where the reference sources exist, the live reference on fresh random scenes.

On x86-64 with glibc (where the fixtures were made) the agreement is bit-exact; elsewhere libm's
sinf/cosf/atanf may differ in the last ulp, so agreement is then checked to 1e-4 relative.
"""
import platform

import numpy as np
import pytest

import golden_util as G
import oracle_bind as ob
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S

EXACT = platform.machine() in ("x86_64", "AMD64")
MODES = {"uni": abi.MODE_REF_UNI, "lt1": abi.MODE_REF_LT1, "bdpt": abi.MODE_REF_BDPT,
         "direct": abi.MODE_REF_DIRECT, "normal": abi.MODE_NORMAL, "position": abi.MODE_POSITION, "lt2": abi.MODE_REF_LT2}
FIXTURES = ["cornell.npz", "furnace.npz", "ico.npz", "soup.npz", "mixture.npz"]


def agree(a, b, rtol=1e-4, frac=0.995):
    if EXACT:
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
    return np.mean(np.all(rel <= rtol, axis=-1)) >= frac


def test_minstd_draws_match_reference_golden(oracle):
    d = G.load("draws.npz")
    for k, v in d.items():
        seed = int(k.split("_")[1])
        a = np.zeros(64, np.float32)
        oracle.o_minstd_draws(seed & 0xFFFFFFFF, 64, ob.ptr(a))
        assert np.array_equal(a.view(np.uint32), v.view(np.uint32)), k


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_hits_match_reference_golden(oracle, name):
    d = G.load(name)
    osc = ob.OracleScene(G.scene_from(d))
    w, h = int(d["width"]), int(d["height"])
    rays = osc.camera_rays(w, h)
    if EXACT:
        assert np.array_equal(rays.view(np.uint32), d["rays"].view(np.uint32))
    hits = osc.trace_closest(d["rays"])
    assert np.array_equal(hits["mesh"], d["hit_mesh"])
    assert np.array_equal(hits["tri"], d["hit_tri"])
    assert np.array_equal(hits["t"].view(np.uint32), d["hit_t"].view(np.uint32))
    valid = d["hit_mesh"] >= 0
    assert np.array_equal(hits["normal"][valid].view(np.uint32), d["hit_normal"][valid].view(np.uint32))
    # the brute-force layout agrees on every hit distance (ties on shared edges may pick the
    # other triangle, since the two layouts visit triangles in different orders)
    lin = osc.trace_closest(d["rays"], use_bvh=False)
    assert np.array_equal(lin["t"].view(np.uint32), d["hit_t"].view(np.uint32))
    assert np.mean(lin["tri"] == d["hit_tri"]) > 0.99


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_paths_match_reference_golden(oracle, name):
    d = G.load(name)
    osc = ob.OracleScene(G.scene_from(d))
    w, h = int(d["width"]), int(d["height"])
    for mname, mode in MODES.items():
        key = "rad_" + mname
        if key not in d:
            continue
        got = osc.render_paths(mode, w, h, d["pixels"], d["seeds"])
        assert agree(got, d[key]), (name, mname)


def test_bsdf_match_reference_golden(oracle):
    d = G.load("bsdf.npz")
    osc = ob.OracleScene(G.scene_from(d))
    i, o, n = d["special_vecs"]
    for mi in range(5):
        dirs, pdf = osc.bsdf_sample(mi, 13, d["n"], d["o"], 1000)
        assert agree(dirs, d[f"dirs_{mi}"]) and agree(pdf[:, None], d[f"pdf_{mi}"][:, None]), mi
        ev = np.array([osc.bsdf_eval(mi, d["n"], d["o"], dd) for dd in d[f"dirs_{mi}"][:200]], np.float32)
        assert agree(ev, d[f"eval_{mi}"]), mi
        assert agree(osc.bsdf_eval(mi, n, o, i)[None], d["special"][mi][None]), mi


def test_material_invariants_like_tst_material(oracle):
    """tst_material.cpp:40-179 on the oracle: pdf >= 0, unit upper-hemisphere samples, validity
    rates, finite non-negative reciprocal BRDF, albedo estimate < 1. The reference's test evaluates
    the BRDF with the unnormalised o = (1,1,1) (:79). With it, cook_torr's Fresnel term is not
    reciprocal (the compiled reference fails that check on 151 of 151 valid samples), while with a
    normalised o oren_nayar's tan(beta) = sin(beta) / cos(theta_o) (material.cpp:157) is not (200
    of 200). So cook_torr is checked with the normalised o, oren_nayar with (1,1,1), each the
    way in which the reference itself passes."""
    d = G.load("bsdf.npz")
    osc = ob.OracleScene(G.scene_from(d))
    n, o = d["n"], d["o"]
    # validity: cook_torr r=0.2 >= 0.8 (:109-116), oren_nayar == 1 (:118-125); the BRDF checks
    # (:127-137) use cook_torr r=0.25 (material 0) and oren_nayar (material 2)
    for mi, min_valid in [(0, 0.0), (1, 0.8), (2, 1.0)]:
        dirs, pdf = osc.bsdf_sample(mi, 13, n, o, 1000)
        assert np.all(pdf >= 0)
        ok = ~np.all(np.abs(dirs) <= 1e-5, axis=1)
        assert np.all(np.abs(np.linalg.norm(dirs[ok], axis=1) - 1) <= 1e-5)
        assert np.all(dirs[ok] @ n >= 0)
        assert ok.mean() >= min_valid
        if mi == 1:
            continue
        acc = np.zeros(3)
        oo = o if mi == 0 else np.ones(3, np.float32)
        for dd, p in zip(dirs[ok], pdf[ok]):
            f = osc.bsdf_eval(mi, n, oo, dd)
            assert np.all(np.isfinite(f)) and np.all(f >= 0)
            fr = osc.bsdf_eval(mi, n, dd, oo)
            assert np.all(np.abs(f - fr) <= 1e-5)
            acc += f * float(n @ dd) / p
        assert np.all(acc / ok.sum() < 1.0)


def test_furnace_oracle_expectation(oracle):
    """tst_pathtracer.cpp:58-86: inward sphere, Lambert 0.7, emission 1: E[sum RGB] = 10."""
    d = G.load("furnace.npz")
    osc = ob.OracleScene(G.scene_from(d))
    rng = np.random.default_rng(3)
    px = rng.integers(0, 32 * 32, 10).repeat(2048).astype(np.uint32)
    seeds = np.array([ob.oracle().o_path_seed(13, int(p), k) for k, p in enumerate(px)], np.uint32)
    for mode in (abi.MODE_REF_UNI, abi.MODE_REF_LT1, abi.MODE_MIS):
        rad = osc.render_paths(mode, 32, 32, px, seeds)
        assert np.all(rad > 0)
        assert abs(rad.sum(axis=1).mean() - 10.0) < 0.3, mode


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_live_reference(reference, seed):
    sc = S.soup(1500 * seed, seed=seed, width=40, height=30)
    osc, rsc = ob.OracleScene(sc), ob.RefScene(sc)
    rays = rsc.camera_rays(40, 30)
    ho, hr = osc.trace_closest(rays), rsc.trace_closest(rays)
    assert np.array_equal(ho["tri"], hr["tri"]) and np.array_equal(ho["mesh"], hr["mesh"])
    rng = np.random.default_rng(seed)
    # random rays from inside the room, including grazing ones
    o = rng.uniform(-1.2, 1.2, (4000, 3)).astype(np.float32)
    dd = rng.normal(size=(4000, 3)).astype(np.float32)
    dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    rr = ob.rays_array(o, dd)
    ho, hr = osc.trace_closest(rr), rsc.trace_closest(rr)
    assert np.array_equal(ho["tri"], hr["tri"]) and np.array_equal(ho["t"].view(np.uint32), hr["t"].view(np.uint32))
    tmin = np.full(4000, 1e-4, np.float32)
    tmax = rng.uniform(0.01, 3.0, 4000).astype(np.float32)
    assert np.array_equal(osc.trace_any(rr, tmin, tmax), rsc.trace_any(rr, tmin, tmax))
    px = rng.integers(0, 1200, 300).astype(np.uint32)
    seeds = rng.integers(0, 2**31 - 1, 300).astype(np.uint32)
    for mode in (abi.MODE_REF_UNI, abi.MODE_REF_LT1, abi.MODE_REF_BDPT, abi.MODE_REF_DIRECT, abi.MODE_REF_LT2):
        a = osc.render_paths(mode, 40, 30, px, seeds)
        b = rsc.render_paths(mode, 40, 30, px, seeds)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), mode


def test_renderer_matches_reference_golden(oracle):
    """pt_image_renderer::render with one thread (renderer.cpp:35-166), the reference's own
    sequential stream and its firefly clamp (renderer.cpp:46-83): the oracle reproduces the
    compositor's buffer bit for bit, and the clamp changes the image."""
    d = G.load("renderer.npz")
    osc = ob.OracleScene(G.scene_from(d))
    w, h, spp = int(d["width"]), int(d["height"]), int(d["spp"])
    for name, mode in (("lt1", abi.MODE_REF_LT1), ("uni", abi.MODE_REF_UNI)):
        for ff in (0, 1):
            got = osc.render_task(mode, w, h, spp, firefly=bool(ff))
            assert np.array_equal(got, d[f"img_{name}_ff{ff}"]), (name, ff)
    assert not np.array_equal(d["img_uni_ff0"], d["img_uni_ff1"])


def test_firefly_clamp_rule(oracle):
    """The clamp on a hand-made image: an interior pixel brighter than all 8 neighbours by more
    than 1.5 in squared norm is capped per channel at their mean squared norm + 1.5; a pixel
    with one neighbour as bright, and border pixels, pass unchanged."""
    est = np.full((5, 6, 3), 0.5, np.float32)
    est[2, 2] = (3.0, 0.2, 1.0)   # squared norm 10.04 > 0.75 + 1.5 against every neighbour
    est[0, 4] = (9.0, 9.0, 9.0)   # border
    est[3, 4] = (2.0, 2.0, 2.0)   # interior, but its neighbour (3, 5) is as bright
    est[3, 5] = (2.0, 2.0, 2.0)   # border
    acc = np.zeros_like(est)
    ob.firefly_add(est, acc)
    cap = np.float32(0.125) * np.float32(8 * 0.75) + np.float32(1.5)
    assert np.allclose(acc[2, 2], np.minimum(est[2, 2], cap))
    assert acc[2, 2, 0] == cap and acc[2, 2, 1] == np.float32(0.2)
    keep = np.ones((5, 6), bool)
    keep[2, 2] = False
    assert np.array_equal(acc[keep], est[keep])


@pytest.mark.parametrize("mode", [abi.MODE_REF_LT1, abi.MODE_REF_UNI, abi.MODE_REF_DIRECT, abi.MODE_REF_BDPT,
                                  abi.MODE_NORMAL])
def test_renderer_matches_live_reference(reference, mode):
    d = G.load("furnace.npz")
    sc = G.scene_from(d)
    osc, rsc = ob.OracleScene(sc), ob.RefScene(sc)
    for ff in (False, True):
        a = osc.render_task(mode, 24, 20, 3, firefly=ff)
        b, _, taken = rsc.render(mode, 24, 20, 3, 1, firefly=ff)
        assert taken == 3 and np.array_equal(a.view(np.uint32), b.view(np.uint32)), ff


def test_compositor_matches_reference_golden(oracle):
    """clamp_compositor and aces_compositor (compositor.cpp:29-98), auto and fixed exposure: the
    oracle's restatement reproduces the reference's 8-bit frame exactly."""
    d = G.load("composite.npz")
    for tm, tname in ((abi.TONEMAP_CLAMP, "clamp"), (abi.TONEMAP_ACES, "aces")):
        for auto in (True, False):
            got = ob.composite(d["image"], tm, auto, 0.8)
            assert np.array_equal(got, d[f"{tname}_{'auto' if auto else 'fixed'}"]), (tname, auto)


def test_compositor_matches_live_reference(reference):
    rng = np.random.default_rng(11)
    img = rng.gamma(0.7, 1.5, (64, 48, 4)).astype(np.float32)
    img[::7, ::5] = 0.0
    for tm in (abi.TONEMAP_CLAMP, abi.TONEMAP_ACES):
        for auto in (True, False):
            assert np.array_equal(ob.composite(img, tm, auto, 1.7), ob.composite(img, tm, auto, 1.7, lib=reference))


def test_transform_matches_reference_golden(oracle):
    """trimesh::transform (geometry.cpp:76-87): positions (m (p, 1)).cart() and normals through
    the reference's cofactor inverse with its w divide; a matrix with |det| <= 1e-5 is refused
    as the reference's "matrix not invertible"."""
    d = G.load("transform.npz")
    for k, m in enumerate(d["mats"]):
        r = ob.transform_mesh(m, d["pos"], d["nrm"])
        if not d["ok"][k]:
            assert r is None, k
            continue
        assert r is not None, k
        assert np.array_equal(r[0].view(np.uint32), d["pos_out"][k].view(np.uint32)), k
        assert np.array_equal(r[1].view(np.uint32), d["nrm_out"][k].view(np.uint32)), k


def test_transform_matches_live_reference(reference):
    rng = np.random.default_rng(5)
    pos = rng.uniform(-10, 10, (200, 3)).astype(np.float32)
    nrm = rng.normal(0, 1, (200, 3)).astype(np.float32)
    for k in range(20):
        m = (np.eye(4) * rng.uniform(0.3, 3.0) + rng.normal(0, 0.5, (4, 4))).astype(np.float32)
        if k % 2 == 0:
            m[3] = (0, 0, 0, 1)  # affine
        a = ob.transform_mesh(m, pos, nrm)
        b = ob.transform_mesh(m, pos, nrm, lib=reference)
        assert (a is None) == (b is None)
        if a is not None:
            assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32)), k
            assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32)), k
