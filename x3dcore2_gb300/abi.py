"""ctypes mirror of include/e8g.h and the loader of the in-tree native library.

The native library (libe8g.so, built by x3dcore2_gb300.build) holds the CUDA kernels and the
C++ host code. There is no fallback: if the library is missing, loading raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# E8G_LIBRARY selects another build of the library (the bounds-checked libe8g_checks.so).
LIB_PATH = os.environ.get("E8G_LIBRARY") or os.path.join(HERE, "libe8g.so")

# status codes
E8G_OK = 0
STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARG", 2: "CUDA", 3: "OUT_OF_MEMORY", 4: "NO_SCENE", 5: "NOT_BUILT",
    6: "UNSUPPORTED", 7: "TIMEOUT", 8: "INTERNAL", 9: "NO_DEVICE", 10: "CANCELLED",
}

# materials
MAT_FAIL_SAFE, MAT_OREN_NAYAR, MAT_COOK_TORR, MAT_MIXTURE = 0, 1, 2, 3
# integrator modes
MODE_REF_UNI, MODE_REF_LT1, MODE_MIS, MODE_REF_BDPT, MODE_BDPT_POWER = 0, 1, 2, 3, 4
MODE_REF_DIRECT, MODE_NORMAL, MODE_POSITION, MODE_REF_LT2 = 5, 6, 7, 8
INTEGRATOR_MEGAKERNEL, INTEGRATOR_WAVEFRONT, INTEGRATOR_PLAIN = 0, 1, 2
RNG_MINSTD, RNG_PHILOX = 0, 1
BVH_SAH, BVH_REFERENCE, BVH_WIDE, BVH_LINEAR = 0, 1, 2, 3
BUILDER_HOST, BUILDER_DEVICE = 0, 1
# compositing
TONEMAP_CLAMP, TONEMAP_ACES = 0, 1
XFORM_REFERENCE, XFORM_NORMALS_AS_DIRECTIONS = 0, 1
COMMIT_REFIT, COMMIT_REBUILD = 0, 1
# generators
GEN_CORNELL, GEN_DISPLACED_ICO, GEN_SOUP, GEN_FURNACE = 0, 1, 2, 3


class Material(C.Structure):
    _fields_ = [("type", C.c_uint32), ("albedo", C.c_float * 3), ("roughness", C.c_float),
                ("ior_re", C.c_float), ("ior_im", C.c_float), ("mix0", C.c_int32),
                ("mix1", C.c_int32), ("ratio", C.c_float)]


class Light(C.Structure):
    _fields_ = [("mesh", C.c_uint32), ("radiance", C.c_float * 3)]


class Camera(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("rot", C.c_float * 9), ("sensor_size", C.c_float),
                ("focal_len", C.c_float), ("aspect", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("num_meshes", C.c_uint32),
                ("mesh_vert_offset", C.POINTER(C.c_uint32)),
                ("mesh_tri_offset", C.POINTER(C.c_uint32)),
                ("mesh_material", C.POINTER(C.c_int32)),
                ("positions", C.POINTER(C.c_float)),
                ("normals", C.POINTER(C.c_float)),
                ("triangles", C.POINTER(C.c_uint32)),
                ("num_materials", C.c_uint32),
                ("materials", C.POINTER(Material)),
                ("num_lights", C.c_uint32),
                ("lights", C.POINTER(Light)),
                ("camera", Camera)]


class BvhOpts(C.Structure):
    _fields_ = [("max_leaf_prims", C.c_uint32), ("num_bins", C.c_uint32), ("tri_cost", C.c_float),
                ("node_cost", C.c_float), ("num_threads", C.c_uint32), ("layout", C.c_uint32),
                ("builder", C.c_uint32)]


class BvhStats(C.Structure):
    _fields_ = [("num_nodes", C.c_uint32), ("num_leaves", C.c_uint32), ("max_depth", C.c_uint32),
                ("num_tris", C.c_uint32), ("avg_leaf_depth", C.c_double), ("build_ms", C.c_double),
                ("node_bytes", C.c_uint64), ("tri_bytes", C.c_uint64), ("layout", C.c_uint32)]


class Ray(C.Structure):
    _fields_ = [("o", C.c_float * 3), ("d", C.c_float * 3)]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("mesh", C.c_int32), ("tri", C.c_int32), ("b1", C.c_float),
                ("b2", C.c_float)]


class RenderParams(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("integrator", C.c_uint32), ("rng", C.c_uint32),
                ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("seed", C.c_uint64), ("max_depth", C.c_uint32), ("rr_start", C.c_uint32),
                ("rr_prob", C.c_float), ("bdpt_max_len", C.c_uint32), ("firefly", C.c_uint32),
                ("sample_offset", C.c_uint32)]


class RenderStats(C.Structure):
    _fields_ = [("ms", C.c_double), ("kernel_ms", C.c_double), ("paths", C.c_uint64),
                ("rays", C.c_uint64), ("nodes", C.c_uint64), ("tris", C.c_uint64),
                ("launches", C.c_uint32), ("counted", C.c_uint32), ("trace_ms", C.c_double),
                ("shade_ms", C.c_double), ("trace_launches", C.c_uint32), ("pad_", C.c_uint32)]


class BatchItem(C.Structure):
    _fields_ = [("scene", C.POINTER(SceneDesc)), ("params", RenderParams),
                ("rgba_out", C.POINTER(C.c_float))]


class TuneResult(C.Structure):
    _fields_ = [("capacity", C.c_uint32), ("bounces_per_graph", C.c_uint32), ("threshold", C.c_uint32),
                ("num_candidates", C.c_uint32), ("cand_capacity", C.c_uint32 * 64),
                ("cand_bounces", C.c_uint32 * 64), ("cand_threshold", C.c_uint32 * 64),
                ("cand_ms", C.c_double * 64), ("shade_variant", C.c_uint32), ("num_shade", C.c_uint32),
                ("shade_ms", C.c_double * 8), ("from_cache", C.c_uint32), ("concurrent", C.c_uint32),
                ("concurrent_ms", C.c_double * 2)]


class GenOpts(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("seed", C.c_uint64), ("level", C.c_uint32),
                ("num_tris", C.c_uint32), ("num_materials", C.c_uint32), ("amplitude", C.c_float),
                ("roughness_lo", C.c_float), ("roughness_hi", C.c_float), ("width", C.c_uint32),
                ("height", C.c_uint32)]


_P = C.c_void_p
_U32 = C.c_uint32
_ST = C.c_int

# name -> (restype, argtypes); every symbol include/e8g.h declares
class MeshData(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32),
                ("positions", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
                ("texcoords", C.POINTER(C.c_float)), ("triangles", C.POINTER(C.c_uint32))]


class PipelineConfig(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("layout", C.c_uint32), ("samples_per_frame", C.c_uint32),
                ("firefly_filter", C.c_uint32), ("auto_exposure", C.c_uint32), ("exposure", C.c_float),
                ("num_threads", C.c_uint32), ("progressive", C.c_uint32), ("integrator", C.c_uint32),
                ("seed", C.c_uint64)]


class CompositeParams(C.Structure):
    _fields_ = [("tonemap", C.c_uint32), ("auto_exposure", C.c_uint32), ("exposure", C.c_float)]


SIGNATURES = {
    "e8g_create": (_ST, [C.POINTER(_P), _P]),
    "e8g_destroy": (_ST, [_P]),
    "e8g_last_error": (C.c_char_p, [_P]),
    "e8g_version": (C.c_char_p, []),
    "e8g_scene_upload": (_ST, [_P, C.POINTER(SceneDesc)]),
    "e8g_scene_build_bvh": (_ST, [_P, C.POINTER(BvhOpts)]),
    "e8g_bvh_get_stats": (_ST, [_P, C.POINTER(BvhStats)]),
    "e8g_default_bvh_opts": (None, [C.POINTER(BvhOpts)]),
    "e8g_bvh_read": (_ST, [_P, _P, _P]),
    "e8g_camera_rays": (_ST, [_P, _U32, _U32, _P]),
    "e8g_trace_closest": (_ST, [_P, _P, _U32, _P]),
    "e8g_trace_any": (_ST, [_P, _P, _P, _P, _U32, _P]),
    "e8g_trace_closest_dev": (_ST, [_P, _P, _U32, _P, _P]),
    "e8g_render": (_ST, [_P, C.POINTER(RenderParams), _P]),
    "e8g_render_dev": (_ST, [_P, C.POINTER(RenderParams), _P, _P]),
    "e8g_render_dev_noalloc": (_ST, [_P, C.POINTER(RenderParams), _P, _P]),
    "e8g_get_render_stats": (_ST, [_P, C.POINTER(RenderStats)]),
    "e8g_set_kernel_timing": (_ST, [_P, C.c_int]),
    "e8g_l2_read_bandwidth": (_ST, [_P, C.c_uint64, _U32, C.POINTER(C.c_double)]),
    "e8g_scene_validate": (_ST, [C.POINTER(SceneDesc), C.c_char_p, C.c_size_t]),
    "e8g_set_memory_limit": (_ST, [_P, C.c_uint64]),
    "e8g_memory_used": (_ST, [_P, C.POINTER(C.c_uint64)]),
    "e8g_cancel": (_ST, [_P]),
    "e8g_progressive_save": (_ST, [_P, _P, C.POINTER(_U32), C.POINTER(_U32), C.POINTER(C.c_uint64)]),
    "e8g_progressive_load": (_ST, [_P, _P, _U32, _U32, C.c_uint64]),
    "e8g_render_progressive": (_ST, [_P, C.POINTER(RenderParams), C.c_int, _P, _P]),
    "e8g_composite": (_ST, [_P, _P, C.c_uint32, C.c_uint32, C.POINTER(CompositeParams), _P]),
    "e8g_composite_dev": (_ST, [_P, _P, C.c_uint32, C.c_uint32, C.POINTER(CompositeParams), _P, _P]),
    "e8g_count_traversal": (_ST, [_P, C.POINTER(RenderParams), C.POINTER(RenderStats)]),
    "e8g_wavefront_tune": (_ST, [_P, C.POINTER(RenderParams), C.POINTER(TuneResult)]),
    "e8g_wavefront_set": (_ST, [_P, _U32, _U32, _U32]),
    "e8g_wavefront_set_shade": (_ST, [_P, _U32]),
    "e8g_wavefront_set_concurrent": (_ST, [_P, C.c_int]),
    "e8g_wavefront_tune_cached": (_ST, [_P, C.POINTER(RenderParams), C.c_char_p, C.POINTER(TuneResult)]),
    "e8g_render_paths": (_ST, [_P, C.POINTER(RenderParams), _P, _P, _U32, _P]),
    "e8g_render_rays": (_ST, [_P, C.POINTER(RenderParams), _P, _U32, _P]),
    "e8g_forward": (_ST, [_P, C.POINTER(RenderParams), _P]),
    "e8g_backward": (_ST, [_P, _P, _P, _P]),
    "e8g_set_materials": (_ST, [_P, C.POINTER(Material), _U32]),
    "e8g_batch_render": (_ST, [_P, C.POINTER(BatchItem), _U32, C.POINTER(RenderStats)]),
    "e8g_default_params": (None, [C.POINTER(RenderParams), _U32, _U32, _U32, _U32]),
    "e8g_path_seed": (_U32, [C.c_uint64, _U32, _U32]),
    "e8g_scene_update_mesh": (_ST, [_P, _U32, _P, _P]),
    "e8g_scene_transform_mesh": (_ST, [_P, _U32, _P, _U32]),
    "e8g_scene_set_camera": (_ST, [_P, C.POINTER(Camera)]),
    "e8g_scene_get_mesh": (_ST, [_P, _U32, _P, _P]),
    "e8g_scene_commit": (_ST, [_P, _U32, C.POINTER(BvhStats)]),
    "e8g_pipeline_config_default": (None, [C.POINTER(PipelineConfig)]),
    "e8g_pipeline_config_set": (_ST, [C.POINTER(PipelineConfig), C.c_char_p, C.c_char_p]),
    "e8g_pipeline_frame": (_ST, [_P, C.POINTER(PipelineConfig), _U32, _U32, _P, _P]),
    "e8g_obj_load": (_ST, [C.c_char_p, C.POINTER(_P), C.c_char_p, C.c_size_t]),
    "e8g_obj_parse": (_ST, [C.c_char_p, C.c_size_t, C.POINTER(_P), C.c_char_p, C.c_size_t]),
    "e8g_host_mesh_data": (_ST, [_P, C.POINTER(MeshData)]),
    "e8g_host_mesh_free": (None, [_P]),
    "e8g_gen_scene": (_ST, [C.POINTER(GenOpts), C.POINTER(_P)]),
    "e8g_host_scene_desc": (_ST, [_P, C.POINTER(SceneDesc)]),
    "e8g_host_scene_free": (None, [_P]),
}

_lib = None


def load(path=None):
    """Load libe8g.so (once). Raises OSError if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"native library {p} is missing: build it with "
                      "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            if path is None:
                raise OSError(f"{p} does not export {name}")
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class E8GError(RuntimeError):
    pass


def check(status, ctx=None, what=""):
    if status != E8G_OK:
        msg = ""
        if ctx is not None:
            err = load().e8g_last_error(ctx)
            msg = err.decode() if err else ""
        raise E8GError(f"{what}: {STATUS_NAMES.get(status, status)} {msg}".strip())
