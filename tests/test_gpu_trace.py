"""Closest-hit and any-hit traversal on the GPU against the reference (golden fixtures) and the
oracle: primitive ids on >= 99.99% of rays, hit distance within 1e-5 relative."""
import numpy as np
import pytest

import golden_util as G
import oracle_bind as ob
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.core import default_params

pytestmark = pytest.mark.gpu

FIXTURES = ["cornell.npz", "furnace.npz", "ico.npz", "soup.npz"]


def compare_hits(g, ref_mesh, ref_tri, ref_t, min_match=0.9999, min_strict=0.999):
    """Ids must match on >= min_match of rays, counting as a match a ray where both sides hit
    at bitwise the same distance (a tie on a shared edge, resolved by visiting order); ids must
    match outright on >= min_strict."""
    same = (g["mesh"] == ref_mesh) & (g["tri"] == ref_tri)
    tie = (~same) & (ref_mesh >= 0) & (g["t"].view(np.uint32) == ref_t.view(np.uint32))
    assert (same | tie).mean() >= min_match, f"id match {(same | tie).mean():.6f}"
    assert same.mean() >= min_strict, f"strict id match {same.mean():.6f}"
    hit = same & (ref_mesh >= 0)
    rel = np.abs(g["t"][hit] - ref_t[hit]) / np.maximum(np.abs(ref_t[hit]), 1e-30)
    assert np.all(rel <= 1e-5), rel.max()
    return same.mean()


@pytest.mark.parametrize("name", FIXTURES)
def test_closest_hits_match_reference_golden_exactly(ctx, name):
    """The reference's tree and visiting order: every id and distance bit-exact, ties included."""
    d = G.load(name)
    ctx.upload(G.scene_from(d), layout=abi.BVH_REFERENCE)
    g = ctx.trace_closest(d["rays"])
    assert np.array_equal(g["mesh"], d["hit_mesh"]) and np.array_equal(g["tri"], d["hit_tri"])
    hit = d["hit_mesh"] >= 0
    assert np.array_equal(g["t"][hit].view(np.uint32), d["hit_t"][hit].view(np.uint32))


@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_WIDE])
@pytest.mark.parametrize("name", FIXTURES)
def test_closest_hits_match_reference_golden_sah(ctx, name, layout):
    """The fast trees (SAH pairs, eight-wide): same hits; ties on shared edges may resolve to the
    other triangle."""
    d = G.load(name)
    ctx.upload(G.scene_from(d), layout=layout)
    assert ctx.bvh_stats()["layout"] == layout
    g = ctx.trace_closest(d["rays"])
    compare_hits(g, d["hit_mesh"], d["hit_tri"], d["hit_t"], min_match=1.0)
    hit = (d["hit_mesh"] >= 0) & (g["mesh"] == d["hit_mesh"])
    assert np.array_equal(g["t"][hit].view(np.uint32), d["hit_t"][hit].view(np.uint32))


@pytest.mark.parametrize("name", FIXTURES)
def test_camera_rays_match_reference_golden(ctx, name):
    d = G.load(name)
    ctx.upload(G.scene_from(d))
    r = ctx.camera_rays(int(d["width"]), int(d["height"]))
    assert np.allclose(r, d["rays"], rtol=0, atol=2e-7)


def random_rays(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    dd = rng.normal(size=(n, 3)).astype(np.float32)
    dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    # a few axis-aligned and degenerate-component directions
    dd[:64] = np.eye(3, dtype=np.float32)[np.arange(64) % 3] * np.where(np.arange(64) % 2, 1, -1)[:, None]
    return ob.rays_array(o, dd)


@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_REFERENCE, abi.BVH_WIDE])
@pytest.mark.parametrize("kind,size", [("ico", 6), ("soup", 100_000), ("ico", 7)])
def test_closest_and_any_hit_match_oracle_on_large_scenes(ctx, kind, size, layout):
    sc = (S.displaced_icosphere(level=size, seed=2, num_materials=64, width=64, height=36) if kind == "ico"
          else S.soup(size, seed=4, width=64, height=64))
    ctx.upload(sc, layout=layout)
    osc = ob.OracleScene(sc)
    rays = random_rays(20000, -1.0, 1.0, seed=size)
    g = ctx.trace_closest(rays)
    o = osc.trace_closest(rays)
    compare_hits(g, o["mesh"], o["tri"], o["t"])
    tmin = np.full(len(rays), 1e-4, np.float32)
    tmax = np.random.default_rng(1).uniform(1e-3, 2.5, len(rays)).astype(np.float32)
    ga = ctx.trace_any(rays, tmin, tmax)
    oa = osc.trace_any(rays, tmin, tmax)
    assert np.mean(ga == oa) >= 0.9999


def test_trace_edge_cases(ctx):
    sc = S.cornell(32, 32)
    ctx.upload(sc)
    osc = ob.OracleScene(sc)
    # empty batch
    assert ctx.trace_closest(np.zeros((0, 6), np.float32))["t"].shape == (0,)
    # rays starting on a wall, grazing along walls, pointing out of the box, and beyond t=1000
    o = np.array([[0.5, 0.0, 0.5], [0.0, 0.5, 0.5], [0.5, 0.5, 0.5], [0.5, 0.5, 0.5], [0.5, 0.5, -2000.0],
                  [1e-7, 0.5, 0.5], [0.5, 1.0, 0.5]], np.float32)
    d = np.array([[0, 1, 0], [0, 1, 0], [0, 0, 1], [0, 0, -1], [0, 0, 1], [0, 0, -1], [0, -1, 0]], np.float32)
    rays = ob.rays_array(o, d)
    g, r = ctx.trace_closest(rays), osc.trace_closest(rays)
    # rays 0 and 6 hit the centre of a quad, on its diagonal: a tie both layouts may resolve
    # differently from the oracle; the distance is the same bits either way
    assert np.array_equal(g["mesh"], r["mesh"])
    assert np.array_equal(g["t"].view(np.uint32), r["t"].view(np.uint32))
    assert g["mesh"][4] == -1  # nothing within 1000
    ctx.upload(sc, layout=abi.BVH_REFERENCE)
    g = ctx.trace_closest(rays)
    assert np.array_equal(g["tri"], r["tri"])


def test_trace_without_scene_is_an_error(lib):
    from x3dcore2_gb300.core import Context
    from x3dcore2_gb300.abi import E8GError
    with Context(0) as c:
        with pytest.raises(E8GError, match="NO_SCENE"):
            c.trace_closest(np.zeros((1, 6), np.float32))


@pytest.mark.parametrize("name", FIXTURES)
def test_linear_layout_matches_the_reference_linear_path_space(ctx, name):
    """E8G_BVH_LINEAR against the oracle's restatement of linear_path_space_layout
    (pathspace.cpp:36-114): every hit's mesh, triangle, distance and barycentrics bit for bit,
    ties included (both keep the first triangle in mesh order), and every any-hit answer."""
    d = G.load(name)
    sc = G.scene_from(d)
    ctx.upload(sc, layout=abi.BVH_LINEAR)
    st = ctx.bvh_stats()
    assert st["layout"] == abi.BVH_LINEAR and st["num_nodes"] == 0
    osc = ob.OracleScene(sc)
    rng = np.random.default_rng(4)
    lo, hi = sc.pos.min(0), sc.pos.max(0)
    dirs = rng.normal(0, 1, (4000, 3))
    rays = np.concatenate([d["rays"], ob.rays_array(rng.uniform(lo, hi, (4000, 3)).astype(np.float32),
                                                    (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32))])
    g = ctx.trace_closest(rays)
    o = osc.trace_closest(rays, use_bvh=False)
    assert np.array_equal(g["mesh"], o["mesh"]) and np.array_equal(g["tri"], o["tri"])
    hit = o["mesh"] >= 0
    assert np.array_equal(g["t"][hit].view(np.uint32), o["t"][hit].view(np.uint32))
    assert np.array_equal(g["b"][hit].view(np.uint32), o["b"][hit].view(np.uint32))
    tmax = np.full(len(rays), 2.0, np.float32)
    assert np.array_equal(ctx.trace_any(rays, 1e-4, tmax), osc.trace_any(rays, np.full(len(rays), 1e-4, np.float32), tmax,
                                                                          use_bvh=False))


def test_linear_layout_renders_like_the_trees(ctx):
    sc = S.cornell(40, 32)
    p = default_params(abi.MODE_REF_LT1, 40, 32, 4, seed=2)
    ctx.upload(sc, layout=abi.BVH_REFERENCE)
    want = ctx.render(p)
    ctx.upload(sc, layout=abi.BVH_LINEAR)
    got = ctx.render(p)
    close = np.abs(got - want) <= np.maximum(1e-4 * np.abs(want), 1e-5)
    assert close.mean() >= 0.999
