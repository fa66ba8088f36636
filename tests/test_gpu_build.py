"""The device BVH builder (E8G_BUILDER_DEVICE: Morton order, PLOC clustering, SAH leaf collapse)
against the host builder and brute force.

The bar: every triangle appears exactly once; every node box is the exact union of its triangles
pushed out as the host builder pushes them out (bit for bit); hits equal the host-built tree's
(distances bit for bit, ids but for ties) and the oracle's brute force; the build is
deterministic; images equal the host-built tree's up to the order of float accumulation."""
import numpy as np
import pytest

import oracle_bind as ob
from test_gpu_trace import compare_hits
from test_gpu_update import pair_boxes_expected, random_rays, same_image, same_paths, split_pairs, with_vertices
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.core import Context, default_params

pytestmark = pytest.mark.gpu

SCENES = {
    "cornell": lambda: S.cornell(48, 40),
    "soup": lambda: S.soup(5000, seed=3, width=64, height=64),
    "ico": lambda: S.displaced_icosphere(level=5, seed=4, num_materials=16, width=96, height=54),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_device_build_is_a_valid_tree(ctx, name):
    sc = SCENES[name]()
    ctx.upload(sc, layout=abi.BVH_SAH, builder=abi.BUILDER_DEVICE)
    st = ctx.bvh_stats()
    assert st["layout"] == abi.BVH_SAH and st["max_depth"] <= 32 and st["num_leaves"] >= 1
    nodes, tris = ctx.bvh_read()
    lo, hi = split_pairs(nodes)
    ids = tris[:, 3].view(np.uint32)
    assert np.array_equal(np.sort(ids), np.arange(sc.num_tris, dtype=np.uint32))
    count = hi[:, 3].view(np.uint32)
    assert count.max() <= 8 and count.sum() == sc.num_tris
    elo, ehi, tv = pair_boxes_expected(sc, sc.pos, lo, hi, tris)
    assert np.array_equal(lo[:, :3].view(np.uint32), elo.view(np.uint32))
    assert np.array_equal(hi[:, :3].view(np.uint32), ehi.view(np.uint32))
    v = tv[ids]
    assert np.array_equal(tris[:, 0:3], v[:, 0])
    assert np.array_equal(tris[:, 4:7], (v[:, 1] - v[:, 0]).astype(np.float32))


def test_device_build_is_deterministic(ctx):
    sc = SCENES["ico"]()
    ctx.upload(sc, builder=abi.BUILDER_DEVICE)
    a = ctx.bvh_read()
    ctx.upload(sc, builder=abi.BUILDER_DEVICE)
    b = ctx.bvh_read()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_WIDE])
@pytest.mark.parametrize("name", ["soup", "ico"])
def test_device_build_hits_equal_host_build(ctx, name, layout):
    sc = SCENES[name]()
    ctx.upload(sc, layout=layout, builder=abi.BUILDER_DEVICE)
    assert ctx.bvh_stats()["layout"] == layout
    rays = np.concatenate([ctx.camera_rays(64, 48), random_rays(sc, 20000, 2)])
    got = ctx.trace_closest(rays)
    with Context(0) as host:
        host.upload(sc, layout=layout)
        want = host.trace_closest(rays)
        occ_d = ctx.trace_any(rays, 1e-4, 3.0)
        occ_h = host.trace_any(rays, 1e-4, 3.0)
    compare_hits(got, want["mesh"], want["tri"], want["t"], min_match=1.0)
    assert np.array_equal(occ_d, occ_h)
    brute = ob.OracleScene(sc).trace_closest(rays, use_bvh=False)
    assert np.array_equal(got["mesh"] >= 0, brute["mesh"] >= 0)


@pytest.mark.parametrize("n", [1, 2, 3, 17])
def test_device_build_of_tiny_scenes(ctx, n):
    rng = np.random.default_rng(n)
    sc0 = S.soup(max(n, 1), seed=n, width=16, height=16)
    ctx.upload(sc0, builder=abi.BUILDER_DEVICE)
    nodes, tris = ctx.bvh_read()
    ids = tris[:, 3].view(np.uint32)
    assert np.array_equal(np.sort(ids), np.arange(sc0.num_tris, dtype=np.uint32))
    rays = random_rays(sc0, 2000, int(rng.integers(100)))
    with Context(0) as host:
        host.upload(sc0)
        want = host.trace_closest(rays)
    compare_hits(ctx.trace_closest(rays), want["mesh"], want["tri"], want["t"], min_match=1.0)


def test_device_build_renders_like_host_build(ctx):
    sc = SCENES["ico"]()
    p = default_params(abi.MODE_MIS, 96, 54, 8, seed=5, max_depth=8, rr_start=3)
    ctx.upload(sc, builder=abi.BUILDER_DEVICE)
    got = ctx.render(p)
    with Context(0) as host:
        host.upload(sc)
        want = host.render(p)
        assert same_paths(ctx, host, p) >= 0.999
    assert same_image(got, want)


def test_device_rebuild_after_transform(ctx):
    """commit(REBUILD) with the device builder needs no host copy of the vertices."""
    sc = SCENES["ico"]()
    ctx.upload(sc, builder=abi.BUILDER_DEVICE)
    c, s = np.cos(0.4), np.sin(0.4)
    m = np.array([[c, -s, 0, 0.1], [s, c, 0, 0], [0, 0, 1, 0.2], [0, 0, 0, 1]], np.float32)
    for mesh in range(0, len(sc.mesh_mat), 3):
        ctx.transform_mesh(mesh, m)
    st = ctx.commit(abi.COMMIT_REBUILD)
    assert st["layout"] == abi.BVH_SAH
    pos, nrm = sc.pos.copy(), sc.nrm.copy()
    for mesh in range(0, len(sc.mesh_mat), 3):
        v0, v1 = sc.voff[mesh], sc.voff[mesh + 1]
        pos[v0:v1], nrm[v0:v1] = ob.transform_mesh(m, sc.pos[v0:v1], sc.nrm[v0:v1])
    sc2 = with_vertices(sc, pos, nrm)
    rays = random_rays(sc2, 20000, 7)
    got = ctx.trace_closest(rays)
    with Context(0) as host:
        host.upload(sc2)
        want = host.trace_closest(rays)
    compare_hits(got, want["mesh"], want["tri"], want["t"], min_match=1.0)


@pytest.fixture(scope="module")
def collapse_checker(tmp_path_factory):
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    csrc = os.path.join(root, "x3dcore2_gb300", "csrc")
    exe = tmp_path_factory.mktemp("collapse") / "wide_collapse_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-pthread", f"-I{csrc}",
                    f"-I{os.path.join(root, 'include')}", os.path.join(root, "tests", "cpp", "wide_collapse_check.cpp"),
                    os.path.join(csrc, "bvh.cpp"), os.path.join(csrc, "bvh_wide.cpp"), "-o", str(exe)],
                   check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("name", ["soup", "ico"])
def test_device_wide_collapse_equals_host_collapse(ctx, collapse_checker, tmp_path, name):
    """The eight-wide collapse on the device writes, byte for byte, the nodes and triangle order
    the host collapse (bvh_wide.cpp) writes for the same binary tree."""
    import subprocess
    from test_wide_bvh import dump
    import ctypes as C
    sc = SCENES[name]()

    def opts(layout):  # the same binary tree for both layouts: an explicit triangle cost
        o = abi.BvhOpts()
        ctx.lib.e8g_default_bvh_opts(C.byref(o))
        o.layout, o.builder, o.tri_cost = layout, abi.BUILDER_DEVICE, 3.0
        return o
    ctx.upload(sc, build=False)
    ctx.build_bvh(opts(abi.BVH_SAH))
    nodes_b, tris_b = ctx.bvh_read()
    nn = ctx.bvh_stats()["num_nodes"]
    ctx.build_bvh(opts(abi.BVH_WIDE))
    st = ctx.bvh_stats()
    assert st["layout"] == abi.BVH_WIDE
    nodes_w, tris_w = ctx.bvh_read()
    dump(sc, tmp_path / "scene.bin")
    with open(tmp_path / "tree.bin", "wb") as f:
        f.write(np.array([nn], np.uint32).tobytes())
        f.write(nodes_b.tobytes())
        f.write(np.ascontiguousarray(tris_b[:, 3]).view(np.uint32).tobytes())
    cam = np.array(list(sc.camera.origin), np.float32)
    max_abs = np.float32(max(np.abs(sc.pos).max(), np.abs(cam).max()))
    subprocess.run([str(collapse_checker), str(tmp_path / "scene.bin"), str(tmp_path / "tree.bin"), "%.9g" % max_abs,
                    str(tmp_path / "out.bin")], check=True)
    out = np.fromfile(tmp_path / "out.bin", np.uint32)
    ok, wn = int(out[0]), int(out[1])
    assert ok == 1 and wn == st["num_nodes"]
    host_nodes = out[2:2 + 24 * wn]
    host_order = out[2 + 24 * wn:]
    assert np.array_equal(nodes_w.view(np.uint32), host_nodes)
    assert np.array_equal(np.ascontiguousarray(tris_w[:, 3]).view(np.uint32), host_order)


@pytest.mark.parametrize("name", ["soup", "ico"])
def test_refit_of_device_wide_tree_keeps_its_bytes(ctx, name):
    """The refit walks the eight-wide tree level by level from the boundaries its builder recorded;
    on a device-built tree (boundaries from the device collapse) a refit of the unchanged scene
    writes the bytes that build wrote."""
    sc = SCENES[name]()
    ctx.upload(sc, layout=abi.BVH_WIDE, builder=abi.BUILDER_DEVICE)
    assert ctx.bvh_stats()["layout"] == abi.BVH_WIDE
    nodes0, tris0 = ctx.bvh_read()
    st = ctx.commit(abi.COMMIT_REFIT)
    assert st["layout"] == abi.BVH_WIDE
    nodes1, tris1 = ctx.bvh_read()
    assert np.array_equal(nodes0, nodes1)
    assert np.array_equal(tris0.view(np.uint32), tris1.view(np.uint32))
