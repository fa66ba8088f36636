"""Python view of the C ABI: one Context per GPU, owning an uploaded scene and its BVH.

Mirrors the reference's split between scene commit (path space / lights / materials actuators,
corelib/src/pathspace.cpp:292-328) and rendering (pt_image_renderer::render,
corelib/src/renderer.cpp:106-166). Every call goes through libe8g.so; nothing here computes.
"""
import ctypes as C

import numpy as np

from . import abi

_P = C.c_void_p


def _ptr(a):
    return a.ctypes.data_as(_P)


def default_params(mode, width, height, spp, **overrides):
    p = abi.RenderParams()
    abi.load().e8g_default_params(C.byref(p), mode, width, height, spp)
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def pipeline_config(**settings):
    """The pipeline's settings: the reference's defaults, then each name=value as flex_config
    sets it (e8g_pipeline_config_set), e.g. path_tracer="bidirectional_mis", exposure=1.5."""
    lib = abi.load()
    cfg = abi.PipelineConfig()
    lib.e8g_pipeline_config_default(C.byref(cfg))
    for k, v in settings.items():
        if isinstance(v, bool):
            v = "true" if v else "false"
        abi.check(lib.e8g_pipeline_config_set(C.byref(cfg), k.encode(), str(v).encode()),
                  what=f"e8g_pipeline_config_set({k}={v})")
    return cfg


def path_seed(seed, pixel, sample):
    return abi.load().e8g_path_seed(seed, pixel, sample)


class Context:
    def __init__(self, device=0):
        self.lib = abi.load()
        self.h = _P()
        opts = (C.c_int32 * 2)(device, 0)
        st = self.lib.e8g_create(C.byref(self.h), C.cast(opts, _P))
        abi.check(st, None, "e8g_create")
        self.scene = None

    def close(self):
        if self.h:
            self.lib.e8g_destroy(self.h)
            self.h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        abi.check(st, self.h, what)

    # ---- scene commit -------------------------------------------------------------------
    def upload(self, scene, build=True, bvh_opts=None, layout=abi.BVH_SAH, builder=abi.BUILDER_HOST):
        self._check(self.lib.e8g_scene_upload(self.h, C.byref(scene.desc)), "e8g_scene_upload")
        self.scene = scene
        if build:
            self.build_bvh(bvh_opts, layout, builder)
        return self

    def build_bvh(self, opts=None, layout=abi.BVH_SAH, builder=abi.BUILDER_HOST):
        """layout BVH_SAH: the fast tree; BVH_REFERENCE: corelib's own tree and visiting order;
        builder BUILDER_DEVICE builds on the GPU."""
        if opts is None:
            opts = abi.BvhOpts()
            self.lib.e8g_default_bvh_opts(C.byref(opts))
            opts.layout = layout
            opts.builder = builder
        self._check(self.lib.e8g_scene_build_bvh(self.h, C.byref(opts)), "e8g_scene_build_bvh")

    def bvh_stats(self):
        s = abi.BvhStats()
        self._check(self.lib.e8g_bvh_get_stats(self.h, C.byref(s)), "e8g_bvh_get_stats")
        return {k: getattr(s, k) for k, _ in abi.BvhStats._fields_}

    def bvh_read(self):
        """The device tree as (node bytes, triangle records (n, 12) float32)."""
        st = self.bvh_stats()
        nodes = np.zeros(st["node_bytes"], np.uint8)
        tris = np.zeros((st["num_tris"], 12), np.float32)
        self._check(self.lib.e8g_bvh_read(self.h, _ptr(nodes), _ptr(tris)), "e8g_bvh_read")
        return nodes, tris

    def pipeline_frame(self, cfg, width, height, want_rgba=False):
        """One pipeline frame: (8-bit RGBA pixels (h, w, 4), float image or None)."""
        px = np.zeros((height, width, 4), np.uint8)
        rgba = np.zeros((height, width, 4), np.float32) if want_rgba else None
        self._check(self.lib.e8g_pipeline_frame(self.h, C.byref(cfg), width, height, _ptr(px),
                                                None if rgba is None else _ptr(rgba)), "e8g_pipeline_frame")
        return px, rgba

    # ---- incremental updates ------------------------------------------------------------
    def mesh_vertex_count(self, mesh):
        d = self.scene.desc
        return d.mesh_vert_offset[mesh + 1] - d.mesh_vert_offset[mesh]

    def update_mesh(self, mesh, positions, normals=None):
        """New blueprint vertices (and normals) of one mesh; needs commit() before rendering."""
        n = self.mesh_vertex_count(mesh)
        pos = np.ascontiguousarray(positions, np.float32).reshape(n, 3)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(n, 3)
        self._check(self.lib.e8g_scene_update_mesh(self.h, mesh, _ptr(pos), None if nrm is None else _ptr(nrm)),
                    "e8g_scene_update_mesh")

    def transform_mesh(self, mesh, matrix, flags=abi.XFORM_REFERENCE):
        """trimesh::transform of one mesh's blueprint by a 4x4 matrix (row-major), on the device."""
        m = np.ascontiguousarray(matrix, np.float32).reshape(16)
        self._check(self.lib.e8g_scene_transform_mesh(self.h, mesh, _ptr(m), flags), "e8g_scene_transform_mesh")

    def set_camera(self, camera):
        self._check(self.lib.e8g_scene_set_camera(self.h, C.byref(camera)), "e8g_scene_set_camera")

    def get_mesh(self, mesh):
        n = self.mesh_vertex_count(mesh)
        pos = np.zeros((n, 3), np.float32)
        nrm = np.zeros((n, 3), np.float32)
        self._check(self.lib.e8g_scene_get_mesh(self.h, mesh, _ptr(pos), _ptr(nrm)), "e8g_scene_get_mesh")
        return pos, nrm

    def commit(self, mode=abi.COMMIT_REFIT):
        s = abi.BvhStats()
        self._check(self.lib.e8g_scene_commit(self.h, mode, C.byref(s)), "e8g_scene_commit")
        return {k: getattr(s, k) for k, _ in abi.BvhStats._fields_}

    # ---- traversal ----------------------------------------------------------------------
    def camera_rays(self, w, h):
        out = np.empty((w * h, 6), np.float32)
        self._check(self.lib.e8g_camera_rays(self.h, w, h, _ptr(out)), "e8g_camera_rays")
        return out

    def trace_closest(self, rays):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = len(rays)
        raw = np.zeros((n, 5), np.float32)
        self._check(self.lib.e8g_trace_closest(self.h, _ptr(rays), n, _ptr(raw)), "e8g_trace_closest")
        return dict(t=raw[:, 0].copy(), mesh=raw[:, 1].view(np.int32).copy(),
                    tri=raw[:, 2].view(np.int32).copy(), b=raw[:, 3:5].copy())

    def trace_any(self, rays, tmin, tmax):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = len(rays)
        out = np.zeros(n, np.uint8)
        tmin = np.ascontiguousarray(np.broadcast_to(tmin, (n,)), np.float32)
        tmax = np.ascontiguousarray(np.broadcast_to(tmax, (n,)), np.float32)
        self._check(self.lib.e8g_trace_any(self.h, _ptr(rays), _ptr(tmin), _ptr(tmax), n, _ptr(out)),
                    "e8g_trace_any")
        return out

    # ---- rendering ----------------------------------------------------------------------
    def render(self, params):
        out = np.zeros((params.height, params.width, 4), np.float32)
        self._check(self.lib.e8g_render(self.h, C.byref(params), _ptr(out)), "e8g_render")
        return out

    def render_dev(self, params, d_out_ptr, stream=None):
        self._check(self.lib.e8g_render_dev(self.h, C.byref(params), _P(d_out_ptr), _P(stream)),
                    "e8g_render_dev")

    def render_progressive(self, params, d_out_ptr, reset=False, stream=None):
        """e8g_render_progressive: params.spp more samples into the running mean at d_out_ptr."""
        self._check(self.lib.e8g_render_progressive(self.h, C.byref(params), int(reset), _P(d_out_ptr), _P(stream)),
                    "e8g_render_progressive")

    def render_paths(self, params, pixels, samples):
        pixels = np.ascontiguousarray(pixels, np.uint32)
        samples = np.ascontiguousarray(np.broadcast_to(samples, pixels.shape), np.uint32)
        out = np.zeros((len(pixels), 3), np.float32)
        self._check(self.lib.e8g_render_paths(self.h, C.byref(params), _ptr(pixels), _ptr(samples),
                                              len(pixels), _ptr(out)), "e8g_render_paths")
        return out

    def render_rays(self, params, rays):
        """Per-path radiance for explicit primary rays ((n, 6): origin, direction)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        out = np.zeros((len(rays), 3), np.float32)
        self._check(self.lib.e8g_render_rays(self.h, C.byref(params), _ptr(rays), len(rays), _ptr(out)),
                    "e8g_render_rays")
        return out

    def composite(self, rgba, tonemap=abi.TONEMAP_ACES, auto_exposure=True, exposure=1.0):
        """e8g_composite: the reference's compositors on a float (h, w, 4) image -> uint8 RGBA."""
        rgba = np.ascontiguousarray(rgba, np.float32)
        h, w = rgba.shape[:2]
        out = np.zeros((h, w, 4), np.uint8)
        cp = abi.CompositeParams(tonemap, int(auto_exposure), exposure)
        self._check(self.lib.e8g_composite(self.h, _ptr(rgba), w, h, C.byref(cp), _ptr(out)), "e8g_composite")
        return out

    def set_memory_limit(self, nbytes):
        """e8g_set_memory_limit: cap on the context's device memory (0: none)."""
        self._check(self.lib.e8g_set_memory_limit(self.h, int(nbytes)), "e8g_set_memory_limit")

    def memory_used(self):
        """e8g_memory_used: device bytes the context holds."""
        v = C.c_uint64(0)
        self._check(self.lib.e8g_memory_used(self.h, C.byref(v)), "e8g_memory_used")
        return v.value

    def set_kernel_timing(self, on=True):
        """e8g_set_kernel_timing: the wavefront times its trace and shading kernels per bounce."""
        self._check(self.lib.e8g_set_kernel_timing(self.h, int(on)), "e8g_set_kernel_timing")

    def stats(self):
        s = abi.RenderStats()
        self._check(self.lib.e8g_get_render_stats(self.h, C.byref(s)), "e8g_get_render_stats")
        return {k: getattr(s, k) for k, _ in abi.RenderStats._fields_}

    def count_traversal(self, params):
        s = abi.RenderStats()
        self._check(self.lib.e8g_count_traversal(self.h, C.byref(params), C.byref(s)),
                    "e8g_count_traversal")
        return {k: getattr(s, k) for k, _ in abi.RenderStats._fields_}

    # ---- differentiable rendering -------------------------------------------------------
    def forward(self, params):
        out = np.zeros((params.height, params.width, 4), np.float32)
        self._check(self.lib.e8g_forward(self.h, C.byref(params), _ptr(out)), "e8g_forward")
        return out

    def backward(self, dl_dimage):
        nm = self.scene.num_materials
        dl = np.ascontiguousarray(dl_dimage, np.float32)
        da = np.zeros((nm, 3), np.float32)
        dr = np.zeros(nm, np.float32)
        self._check(self.lib.e8g_backward(self.h, _ptr(dl), _ptr(da), _ptr(dr)), "e8g_backward")
        return da, dr

    def set_materials(self, materials):
        arr = (abi.Material * len(materials))(*materials)
        self._check(self.lib.e8g_set_materials(self.h, arr, len(materials)), "e8g_set_materials")


def render_batch(ctx, scenes, params):
    """e8g_batch_render: many scenes in one persistent launch; returns images and stats."""
    n = len(scenes)
    items = (abi.BatchItem * n)()
    outs = []
    for k, (sc, p) in enumerate(zip(scenes, params)):
        img = np.zeros((p.height, p.width, 4), np.float32)
        outs.append(img)
        items[k].scene = C.pointer(sc.desc)
        items[k].params = p
        items[k].rgba_out = img.ctypes.data_as(C.POINTER(C.c_float))
    st = abi.RenderStats()
    abi.check(ctx.lib.e8g_batch_render(ctx.h, items, n, C.byref(st)), ctx.h, "e8g_batch_render")
    return outs, {k: getattr(st, k) for k, _ in abi.RenderStats._fields_}
