"""Failure paths on the GPU, injected on the host (nothing here faults, traps or hangs a GPU):

* a device memory limit on the context (e8g_set_memory_limit) makes uploads, builds and renders
  fail with E8G_ERR_OUT_OF_MEMORY as a failed cudaMalloc would; a failed upload leaves no scene and
  a failed build no tree (the next render reports it), and the context works again once the limit
  is lifted;
* e8g_cancel, before a call or from another thread during a long wavefront render, stops it with
  E8G_ERR_CANCELLED after its kernels in flight, and the context renders normally afterwards;
* a scene with non-finite values is refused before any device work and the previous scene stays;
* degenerate geometry (zero-area and collinear triangles, a mesh without triangles, coincident
  vertices) renders like the oracle's restatement of the reference;
* progressive rendering saved and loaded into a fresh context continues to the same image.
"""
import ctypes as C
import threading
import time

import numpy as np
import pytest

import oracle_bind as ob
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.core import Context, default_params

pytestmark = pytest.mark.gpu


def render_status(lib, ctx, p):
    out = np.zeros((p.height, p.width, 4), np.float32)
    st = lib.e8g_render(ctx.h, C.byref(p), out.ctypes.data_as(C.c_void_p))
    return st, out


def used(lib, ctx):
    v = C.c_uint64()
    assert lib.e8g_memory_used(ctx.h, C.byref(v)) == 0
    return v.value


def test_memory_limit_fails_cleanly_and_recovers(lib):
    sc = S.cornell(256, 256)
    p = default_params(abi.MODE_MIS, 256, 256, 4, seed=5, max_depth=6)
    with Context(0) as ref:
        ref.upload(sc)
        want = ref.render(p)
    with Context(0) as ctx:
        ctx.upload(sc)
        assert used(lib, ctx) > 0
        # the render needs its first-hit cache and accumulator (about 4 MB at 256x256)
        assert lib.e8g_set_memory_limit(ctx.h, used(lib, ctx) + (1 << 20)) == 0
        st, _ = render_status(lib, ctx, p)
        assert st == 3 and b"limit" in lib.e8g_last_error(ctx.h)
        limit_used = used(lib, ctx)
        assert lib.e8g_set_memory_limit(ctx.h, 0) == 0
        st, got = render_status(lib, ctx, p)
        assert st == 0 and used(lib, ctx) > limit_used
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)

        # an upload that does not fit leaves no scene; a build that does not fit leaves no tree
        big = S.displaced_icosphere(level=6, seed=1, num_materials=64, width=256, height=256)
        assert lib.e8g_set_memory_limit(ctx.h, 1 << 20) == 0
        assert lib.e8g_scene_upload(ctx.h, C.byref(big.desc)) == 3
        assert render_status(lib, ctx, p)[0] == 4  # E8G_ERR_NO_SCENE
        assert lib.e8g_set_memory_limit(ctx.h, 0) == 0
        ctx.upload(big, build=False)
        assert lib.e8g_set_memory_limit(ctx.h, used(lib, ctx) + 4096) == 0
        opts = abi.BvhOpts()
        lib.e8g_default_bvh_opts(C.byref(opts))
        assert lib.e8g_scene_build_bvh(ctx.h, C.byref(opts)) == 3
        assert render_status(lib, ctx, p)[0] == 5
        assert lib.e8g_set_memory_limit(ctx.h, 0) == 0
        ctx.build_bvh()
        st, img = render_status(lib, ctx, p)
        assert st == 0 and np.all(np.isfinite(img)) and img[..., :3].sum() > 0


def test_cancel_before_and_during_a_render(lib):
    sc = S.displaced_icosphere(level=6, seed=1, num_materials=64, width=1280, height=720)
    with Context(0) as ctx:
        ctx.upload(sc, layout=abi.BVH_WIDE)
        small = default_params(abi.MODE_MIS, 320, 180, 4, seed=1, max_depth=8, rr_start=3,
                               integrator=abi.INTEGRATOR_WAVEFRONT)
        assert lib.e8g_cancel(ctx.h) == 0
        st, _ = render_status(lib, ctx, small)
        assert st == 10 and b"cancel" in lib.e8g_last_error(ctx.h)
        st, img = render_status(lib, ctx, small)  # the request was consumed
        assert st == 0 and img[..., :3].sum() > 0
        # a long wavefront render (about 900 M paths), cancelled from another thread
        big = default_params(abi.MODE_MIS, 1280, 720, 1024, seed=1, max_depth=8, rr_start=3,
                             integrator=abi.INTEGRATOR_WAVEFRONT)
        render_status(lib, ctx, default_params(abi.MODE_MIS, 1280, 720, 1, seed=1, max_depth=8, rr_start=3,
                                               integrator=abi.INTEGRATOR_WAVEFRONT))  # slots allocated
        timer = threading.Timer(0.15, lambda: lib.e8g_cancel(ctx.h))
        t0 = time.perf_counter()
        timer.start()
        st, _ = render_status(lib, ctx, big)
        dt = time.perf_counter() - t0
        timer.join()
        if st == 0:  # finished before the request arrived; the request then stops the next call
            assert render_status(lib, ctx, small)[0] == 10
        else:
            assert st == 10, lib.e8g_last_error(ctx.h)
        st, img = render_status(lib, ctx, small)
        assert st == 0 and np.all(np.isfinite(img)), dt


def test_non_finite_scene_is_refused_and_the_previous_scene_stays(lib):
    sc = S.cornell(64, 48)
    p = default_params(abi.MODE_REF_LT1, 64, 48, 2, seed=3)
    with Context(0) as ctx:
        ctx.upload(sc)
        before = ctx.render(p)
        pos = sc.pos.copy()
        pos[2, 0] = np.nan
        bad = S.Scene(sc.voff, sc.toff, sc.mesh_mat, pos, sc.nrm, sc.tris, sc.material_list(),
                      list(sc.lights[:sc.num_lights]), sc.camera)
        assert lib.e8g_scene_upload(ctx.h, C.byref(bad.desc)) == 1
        assert b"finite" in lib.e8g_last_error(ctx.h)
        after = ctx.render(p)
        np.testing.assert_allclose(after, before, rtol=1e-5, atol=1e-6)
        m = np.eye(4, dtype=np.float32)
        m[0, 3] = np.inf
        assert lib.e8g_scene_transform_mesh(ctx.h, 1, m.ctypes.data_as(C.c_void_p), 0) == 1


def degenerate_scene():
    """The Cornell room plus a mesh of zero-area triangles (three coincident vertices, and three
    collinear ones), an empty mesh, and a sliver triangle."""
    sc = S.cornell(64, 48)
    meshes = []
    for m in range(len(sc.voff) - 1):
        v0, v1, t0, t1 = sc.voff[m], sc.voff[m + 1], sc.toff[m], sc.toff[m + 1]
        meshes.append(S.Mesh(sc.pos[v0:v1], sc.nrm[v0:v1], sc.tris[t0:t1]))
    p = np.array([[0.3, 0.3, 0.3], [0.3, 0.3, 0.3], [0.3, 0.3, 0.3], [0.2, 0.5, 0.4], [0.4, 0.5, 0.4],
                  [0.6, 0.5, 0.4], [0.5, 0.2, 0.3], [0.5, 0.8, 0.3], [0.5000001, 0.5, 0.3]], np.float32)
    n = np.tile(np.array([[0, 0, 1]], np.float32), (len(p), 1))
    meshes.append(S.Mesh(p, n, np.array([[0, 1, 2], [3, 4, 5], [6, 7, 8]], np.uint32)))
    meshes.append(S.Mesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32)))
    mm = list(sc.mesh_mat) + [0, 0]
    return S.from_meshes(meshes, mm, sc.material_list(), list(sc.lights[:sc.num_lights]), sc.camera)


@pytest.mark.parametrize("layout", [abi.BVH_SAH, abi.BVH_WIDE, abi.BVH_REFERENCE])
def test_degenerate_geometry_renders_like_the_oracle(lib, layout):
    sc = degenerate_scene()
    p = default_params(abi.MODE_REF_LT1, 64, 48, 4, seed=9)
    with Context(0) as ctx:
        ctx.upload(sc, layout=layout)
        img = ctx.render(p)[..., :3]
    ref = ob.OracleScene(sc).render(abi.MODE_REF_LT1, 64, 48, 4, seed=9, policy=ob.REF_POLICY)[..., :3]
    assert np.all(np.isfinite(img))
    close = np.all(np.abs(img - ref) <= np.maximum(1e-4 * np.abs(ref), 1e-6), axis=-1)
    assert close.mean() >= 0.995, close.mean()


def test_progressive_checkpoint_resumes(lib):
    sc = S.cornell(96, 64)
    p = default_params(abi.MODE_MIS, 96, 64, 4, seed=13, max_depth=6)
    import torch
    out = torch.empty((64, 96, 4), dtype=torch.float32, device="cuda")
    with Context(0) as a:
        a.upload(sc)
        a.render_progressive(p, out.data_ptr(), reset=True)
        a.render_progressive(p, out.data_ptr())
        w, h, spp = C.c_uint32(), C.c_uint32(), C.c_uint64()
        assert lib.e8g_progressive_save(a.h, None, C.byref(w), C.byref(h), C.byref(spp)) == 0
        assert (w.value, h.value, spp.value) == (96, 64, 8)
        state = np.zeros((64, 96, 4), np.float32)
        assert lib.e8g_progressive_save(a.h, state.ctypes.data_as(C.c_void_p), C.byref(w), C.byref(h),
                                        C.byref(spp)) == 0
        a.render_progressive(p, out.data_ptr())
        torch.cuda.synchronize()
        straight = out.cpu().numpy()
    with Context(0) as b:
        b.upload(sc)
        assert lib.e8g_progressive_load(b.h, state.ctypes.data_as(C.c_void_p), 96, 64, 8) == 0
        b.render_progressive(p, out.data_ptr())
        torch.cuda.synchronize()
        resumed = out.cpu().numpy()
    np.testing.assert_allclose(resumed, straight, rtol=1e-5, atol=1e-6)
