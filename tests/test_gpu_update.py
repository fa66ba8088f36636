"""Incremental scene updates on the GPU: dirty-only mesh uploads, trimesh::transform on the device
and the tree refit (e8g_scene_update_mesh / _transform_mesh / _commit).

The bar: a refit of an unchanged scene writes exactly the bytes of the host build; after vertices
move, every box is the exact union of its triangles pushed out as the build pushes them out (SAH
pairs: checked bit for bit against numpy; eight-wide: every quantized box contains its triangles);
hits after update + commit equal those of a fresh upload of the changed scene, and images do up
to the order of float accumulation; the
device transform equals the oracle's restatement of trimesh::transform bit for bit."""
import numpy as np
import pytest

import golden_util as G
import oracle_bind as ob
from test_gpu_trace import compare_hits
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.abi import E8GError
from x3dcore2_gb300.core import Context, default_params

pytestmark = pytest.mark.gpu


def with_vertices(sc, pos, nrm=None):
    return S.Scene(sc.voff, sc.toff, sc.mesh_mat, pos, sc.nrm if nrm is None else nrm, sc.tris,
                   sc.material_list(), list(sc.lights[:sc.num_lights]), sc.camera)


def deformed(sc, seed, amp):
    rng = np.random.default_rng(seed)
    return (sc.pos + rng.uniform(-amp, amp, sc.pos.shape)).astype(np.float32)


def random_rays(sc, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = sc.pos.min(0), sc.pos.max(0)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(0, 1, (n, 3))
    return ob.rays_array(o.astype(np.float32), (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32))


def push_all(ctx, sc, pos):
    for m in range(len(sc.mesh_mat)):
        ctx.update_mesh(m, pos[sc.voff[m]:sc.voff[m + 1]])


def same_image(got, want):
    """Equal up to the order of float accumulation (pixels sum their samples with atomics)."""
    close = np.abs(got - want) <= np.maximum(1e-4 * np.abs(want), 1e-5)
    return close.mean() >= 0.999


def same_paths(a, b, p, samples=2):
    """Per-path radiance (no accumulation) of every pixel for `samples` samples: bit-equal on all
    but ties (a ray through a shared edge may pick the other triangle in another tree)."""
    n = p.width * p.height
    pix = np.tile(np.arange(n, dtype=np.uint32), samples)
    smp = np.repeat(np.arange(samples, dtype=np.uint32), n)
    ra, rb = a.render_paths(p, pix, smp), b.render_paths(p, pix, smp)
    eq = np.all(ra.view(np.uint32) == rb.view(np.uint32), axis=1)
    return eq.mean()


def f32(x):
    return np.float32(x)


def pair_boxes_expected(sc, pos, nodes_lo, nodes_hi, tris):
    """Exact unions of every node's triangles pushed out by |v| 1e-6 + eps (float32), children
    before parents (their indices are larger)."""
    nn = len(nodes_lo)
    link = nodes_lo[:, 3].view(np.uint32)
    count = nodes_hi[:, 3].view(np.uint32)
    ids = tris[:, 3].view(np.uint32)
    base = np.repeat(sc.voff[:-1], np.diff(sc.toff)).astype(np.int64)
    tv = pos[sc.tris.astype(np.int64) + base[:, None]]  # (T, 3, 3)
    tlo, thi = tv.min(1), tv.max(1)
    lo = np.zeros((nn, 3), np.float32)
    hi = np.zeros((nn, 3), np.float32)
    for i in range(nn - 1, -1, -1):
        if count[i]:
            sel = ids[link[i]:link[i] + count[i]]
            lo[i], hi[i] = tlo[sel].min(0), thi[sel].max(0)
        else:
            c = link[i]
            lo[i], hi[i] = np.minimum(lo[c], lo[c + 1]), np.maximum(hi[c], hi[c + 1])
    diag = f32(max(f32(tv[..., a].max() - tv[..., a].min()) for a in range(3)))
    eps = f32(diag * f32(1e-6))
    inf_lo = lo - (np.abs(lo) * f32(1e-6) + eps)
    inf_hi = hi + (np.abs(hi) * f32(1e-6) + eps)
    return inf_lo.astype(np.float32), inf_hi.astype(np.float32), tv


def split_pairs(nodes):
    a = nodes.view(np.float32).reshape(2, -1, 4)
    return a[0], a[1]


@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_WIDE])
@pytest.mark.parametrize("which", ["soup", "ico"])
def test_refit_of_unchanged_scene_writes_the_build_bytes(ctx, layout, which):
    sc = S.soup(3000, seed=4) if which == "soup" else S.displaced_icosphere(level=4, seed=2, num_materials=8,
                                                                           width=64, height=36)
    ctx.upload(sc, layout=layout)
    nodes0, tris0 = ctx.bvh_read()
    st = ctx.commit(abi.COMMIT_REFIT)
    assert st["layout"] == layout and st["build_ms"] >= 0
    nodes1, tris1 = ctx.bvh_read()
    assert np.array_equal(nodes0, nodes1)
    assert np.array_equal(tris0.view(np.uint32), tris1.view(np.uint32))


@pytest.mark.parametrize("builder", [abi.BUILDER_HOST, abi.BUILDER_DEVICE])
@pytest.mark.parametrize("n", [1, 2, 9, 40])
def test_refit_of_tiny_wide_trees(ctx, n, builder):
    """Small eight-wide trees (a soup of n triangles in its room: one to three levels): the refit
    of the unchanged scene writes the build's bytes, and after moving every vertex the hits equal
    a fresh build's."""
    sc = S.soup(n, seed=n, width=16, height=16)
    ctx.upload(sc, layout=abi.BVH_WIDE, builder=builder)
    assert ctx.bvh_stats()["layout"] == abi.BVH_WIDE
    nodes0, tris0 = ctx.bvh_read()
    ctx.commit(abi.COMMIT_REFIT)
    nodes1, tris1 = ctx.bvh_read()
    assert np.array_equal(nodes0, nodes1)
    assert np.array_equal(tris0.view(np.uint32), tris1.view(np.uint32))
    pos = deformed(sc, 3, 0.05)
    push_all(ctx, sc, pos)
    ctx.commit(abi.COMMIT_REFIT)
    rays = random_rays(sc, 3000, n)
    with Context(0) as fresh:
        fresh.upload(with_vertices(sc, pos, sc.nrm), layout=abi.BVH_WIDE)
        want = fresh.trace_closest(rays)
    compare_hits(ctx.trace_closest(rays), want["mesh"], want["tri"], want["t"], min_match=1.0)


def test_refit_boxes_after_deformation_are_the_exact_unions(ctx):
    sc = S.soup(2500, seed=6)
    ctx.upload(sc, layout=abi.BVH_SAH)
    pos = deformed(sc, 1, 0.05)
    push_all(ctx, sc, pos)
    ctx.commit(abi.COMMIT_REFIT)
    nodes, tris = ctx.bvh_read()
    lo, hi = split_pairs(nodes)
    elo, ehi, tv = pair_boxes_expected(sc, pos, lo, hi, tris)
    assert np.array_equal(lo[:, :3].view(np.uint32), elo.view(np.uint32))
    assert np.array_equal(hi[:, :3].view(np.uint32), ehi.view(np.uint32))
    ids = tris[:, 3].view(np.uint32)
    v = tv[ids]
    assert np.array_equal(tris[:, 0:3], v[:, 0])
    assert np.array_equal(tris[:, 4:7], (v[:, 1] - v[:, 0]).astype(np.float32))
    assert np.array_equal(tris[:, 8:11], (v[:, 2] - v[:, 0]).astype(np.float32))


def wide_slot_boxes(nodes):
    """Decoded child boxes of every eight-wide node: (N, 8, 3) lo and hi, the slot masks, and each
    node's interior children and leaf triangle ranges."""
    w = nodes.view(np.uint32).reshape(-1, 24)
    org = w[:, 0:3].view(np.float32)
    ex = ((w[:, 3:4] >> (8 * np.arange(3, dtype=np.uint32))) & 0xFF).astype(np.int32) - 127
    step = np.ldexp(1.0, ex)  # (N, 3)
    q = w[:, 8:20].view(np.uint8).reshape(-1, 6, 8).astype(np.float64)  # plane, slot
    lo = org[:, None, :] + q[:, 0:3, :].transpose(0, 2, 1) * step[:, None, :]
    hi = org[:, None, :] + q[:, 3:6, :].transpose(0, 2, 1) * step[:, None, :]
    return w, lo, hi


def test_wide_refit_after_deformation_contains_every_triangle(ctx):
    sc = S.displaced_icosphere(level=4, seed=3, num_materials=8, width=64, height=36)
    ctx.upload(sc, layout=abi.BVH_WIDE)
    assert ctx.bvh_stats()["layout"] == abi.BVH_WIDE
    pos = deformed(sc, 2, 0.02)
    push_all(ctx, sc, pos)
    ctx.commit(abi.COMMIT_REFIT)
    nodes, tris = ctx.bvh_read()
    w, lo, hi = wide_slot_boxes(nodes)
    base = np.repeat(sc.voff[:-1], np.diff(sc.toff)).astype(np.int64)
    tv = pos[sc.tris.astype(np.int64) + base[:, None]].astype(np.float64)
    ids = tris[:, 3].view(np.uint32)
    # exact boxes per node, children first (breadth-first order: children have larger indices)
    n = len(w)
    nlo = np.full((n, 3), np.inf)
    nhi = np.full((n, 3), -np.inf)
    for i in range(n - 1, -1, -1):
        imask, cbase, tbase = int(w[i, 3] >> 24), int(w[i, 4]), int(w[i, 5])
        meta = w[i, 6:8].view(np.uint8)
        counts, leaves = int(w[i, 20]), int(w[i, 21])
        for s in range(8):
            if imask >> s & 1:
                c = cbase + bin(imask & ((1 << s) - 1)).count("1")
                blo, bhi = nlo[c], nhi[c]
            elif leaves >> s & 1:
                k0, cnt = tbase + int(meta[s]), (counts >> (4 * s)) & 15
                t = tv[ids[k0:k0 + cnt]]
                blo, bhi = t.min(axis=(0, 1)), t.max(axis=(0, 1))
            else:
                continue
            assert np.all(lo[i, s] <= blo) and np.all(hi[i, s] >= bhi), (i, s)
            nlo[i] = np.minimum(nlo[i], blo)
            nhi[i] = np.maximum(nhi[i], bhi)


@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_WIDE])
def test_refit_hits_equal_a_fresh_build(ctx, layout):
    sc = S.displaced_icosphere(level=5, seed=7, num_materials=8, width=96, height=54)
    ctx.upload(sc, layout=layout)
    pos = deformed(sc, 3, 0.01)
    push_all(ctx, sc, pos)
    ctx.commit(abi.COMMIT_REFIT)
    sc2 = with_vertices(sc, pos)
    rays = np.concatenate([ctx.camera_rays(96, 54), random_rays(sc2, 20000, 5)])
    got = ctx.trace_closest(rays)
    with Context(0) as fresh:
        fresh.upload(sc2, layout=layout)
        want = fresh.trace_closest(rays)
    compare_hits(got, want["mesh"], want["tri"], want["t"], min_match=1.0)
    brute = ob.OracleScene(sc2).trace_closest(rays, use_bvh=False)
    hit = brute["mesh"] >= 0
    assert np.array_equal(got["mesh"] >= 0, hit)
    rel = np.abs(got["t"][hit] - brute["t"][hit]) / brute["t"][hit]
    assert rel.max() <= 1e-5


def test_dirty_scene_refuses_to_render_until_commit(ctx):
    sc = S.cornell(32, 32)
    ctx.upload(sc)
    ctx.update_mesh(0, sc.pos[sc.voff[0]:sc.voff[1]])
    p = default_params(abi.MODE_MIS, 32, 32, 1)
    with pytest.raises(E8GError, match="NOT_BUILT"):
        ctx.render(p)
    ctx.commit()
    ctx.render(p)


def test_transform_equals_oracle_trimesh_transform(ctx):
    sc = S.displaced_icosphere(level=3, seed=1, num_materials=4, width=32, height=18)
    ctx.upload(sc, layout=abi.BVH_SAH)
    mats = G.load("transform.npz")["mats"]
    mesh = 0
    v0, v1 = sc.voff[mesh], sc.voff[mesh + 1]
    for k, m in enumerate(mats):
        want = ob.transform_mesh(m, sc.pos[v0:v1], sc.nrm[v0:v1])
        if want is None:
            with pytest.raises(E8GError, match="not invertible"):
                ctx.transform_mesh(mesh, m)
            continue
        ctx.transform_mesh(mesh, m)
        pos, nrm = ctx.get_mesh(mesh)
        assert np.array_equal(pos.view(np.uint32), want[0].view(np.uint32)), k
        assert np.array_equal(nrm.view(np.uint32), want[1].view(np.uint32)), k
    # normals as directions: the inverse transpose applied to (n, 0)
    m = mats[2]
    ctx.transform_mesh(mesh, m, abi.XFORM_NORMALS_AS_DIRECTIONS)
    _, nrm = ctx.get_mesh(mesh)
    ninv = np.linalg.inv(m.astype(np.float64)).T[:3, :3]
    want = sc.nrm[v0:v1].astype(np.float64) @ ninv.T
    assert np.allclose(nrm, want, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("mode", [abi.COMMIT_REFIT, abi.COMMIT_REBUILD])
@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_WIDE])
def test_transform_commit_renders_like_an_upload(ctx, mode, layout):
    """A box of the Cornell scene moved by a rigid motion: the image after transform + commit is the
    image of the scene uploaded with the transformed mesh."""
    sc = S.cornell(48, 40)
    light_meshes = {sc.lights[i].mesh for i in range(sc.num_lights)}
    mesh = max(m for m in range(len(sc.mesh_mat)) if m not in light_meshes)
    c, s = np.cos(0.3), np.sin(0.3)
    m = np.array([[c, 0, s, 0.05], [0, 1, 0, 0.02], [-s, 0, c, -0.04], [0, 0, 0, 1]], np.float32)
    ctx.upload(sc, layout=layout)
    ctx.transform_mesh(mesh, m)
    ctx.commit(mode)
    p = default_params(abi.MODE_MIS, 48, 40, 8)
    got = ctx.render(p)
    v0, v1 = sc.voff[mesh], sc.voff[mesh + 1]
    tp, tn = ob.transform_mesh(m, sc.pos[v0:v1], sc.nrm[v0:v1])
    pos, nrm = sc.pos.copy(), sc.nrm.copy()
    pos[v0:v1], nrm[v0:v1] = tp, tn
    with Context(0) as fresh:
        fresh.upload(with_vertices(sc, pos, nrm), layout=layout)
        want = fresh.render(p)
        assert same_paths(ctx, fresh, p) >= 0.999
    assert same_image(got, want)


def test_update_of_a_light_mesh_recomputes_its_power(ctx):
    """A light quad scaled by update_mesh: area, power and light CDF follow, as in an upload."""
    sc = S.cornell(40, 40)
    lm = sc.lights[0].mesh
    v0, v1 = sc.voff[lm], sc.voff[lm + 1]
    pos = sc.pos.copy()
    ctr = pos[v0:v1].mean(0)
    pos[v0:v1] = ctr + (pos[v0:v1] - ctr) * np.float32(1.6)
    ctx.upload(sc)
    ctx.update_mesh(lm, pos[v0:v1])
    ctx.commit(abi.COMMIT_REFIT)
    p = default_params(abi.MODE_REF_LT1, 40, 40, 8)
    got = ctx.render(p)
    with Context(0) as fresh:
        fresh.upload(with_vertices(sc, pos))
        want = fresh.render(p)
        assert same_paths(ctx, fresh, p) >= 0.999
    assert same_image(got, want)
    ctx.upload(sc)  # the power changed: the unchanged scene renders differently
    assert not same_image(ctx.render(p), got)


def test_set_camera_renders_like_an_upload(ctx):
    sc = S.cornell(40, 32)
    ctx.upload(sc)
    cam = abi.Camera.from_buffer_copy(sc.camera)
    cam.origin[0] += 0.1
    cam.origin[2] -= 0.3
    ctx.set_camera(cam)
    p = default_params(abi.MODE_MIS, 40, 32, 4)
    got = ctx.render(p)
    sc2 = S.Scene(sc.voff, sc.toff, sc.mesh_mat, sc.pos, sc.nrm, sc.tris, sc.material_list(),
                  list(sc.lights[:sc.num_lights]), cam)
    with Context(0) as fresh:
        fresh.upload(sc2)
        want = fresh.render(p)
        assert same_paths(ctx, fresh, p) == 1.0
    assert same_image(got, want)


def test_reference_layout_commit_keeps_reference_hit_identities(ctx):
    """The reference layout rebuilds on commit, as the reference does: ids match the reference's
    tree (the oracle's restatement of it) bit for bit after a transform."""
    sc = S.soup(2000, seed=8, width=48, height=48)
    ctx.upload(sc, layout=abi.BVH_REFERENCE)
    m = np.array([[0.9, 0.1, 0, 0.2], [-0.1, 0.9, 0, 0.1], [0, 0, 1.1, -0.3], [0, 0, 0, 1]], np.float32)
    ctx.transform_mesh(0, m)
    ctx.commit(abi.COMMIT_REFIT)
    v0, v1 = sc.voff[0], sc.voff[1]
    tp, tn = ob.transform_mesh(m, sc.pos[v0:v1], sc.nrm[v0:v1])
    pos, nrm = sc.pos.copy(), sc.nrm.copy()
    pos[v0:v1], nrm[v0:v1] = tp, tn
    sc2 = with_vertices(sc, pos, nrm)
    rays = np.concatenate([ctx.camera_rays(48, 48), random_rays(sc2, 5000, 9)])
    got = ctx.trace_closest(rays)
    want = ob.OracleScene(sc2).trace_closest(rays, use_bvh=True)
    assert np.array_equal(got["mesh"], want["mesh"]) and np.array_equal(got["tri"], want["tri"])
    hit = want["mesh"] >= 0
    assert np.array_equal(got["t"][hit].view(np.uint32), want["t"][hit].view(np.uint32))


def test_update_entry_points_refuse_bad_arguments(lib):
    """Error paths: no scene, a mesh out of range, a NULL array, an unknown commit mode or
    transform flag: a status, never a crash."""
    import ctypes as C
    from x3dcore2_gb300 import abi as A
    with Context(0) as c:
        m = np.eye(4, dtype=np.float32)
        assert lib.e8g_scene_commit(c.h, A.COMMIT_REFIT, None) == 4           # E8G_ERR_NO_SCENE
        assert lib.e8g_scene_transform_mesh(c.h, 0, m.ctypes.data, 0) == 4
        sc = S.cornell(16, 16)
        c.upload(sc)
        nm = len(sc.mesh_mat)
        pos = np.zeros((1 << 12, 3), np.float32)
        assert lib.e8g_scene_update_mesh(c.h, nm, pos.ctypes.data, None) == 1  # E8G_ERR_INVALID_ARG
        assert lib.e8g_scene_update_mesh(c.h, 0, None, None) == 1
        assert lib.e8g_scene_transform_mesh(c.h, nm, m.ctypes.data, 0) == 1
        assert lib.e8g_scene_transform_mesh(c.h, 0, m.ctypes.data, 7) == 1
        assert lib.e8g_scene_commit(c.h, 9, None) == 1
        assert lib.e8g_scene_get_mesh(c.h, nm, None, None) == 1
        # nothing changed, so the scene still renders
        c.render(default_params(abi.MODE_MIS, 16, 16, 1))
