"""ctypes bindings of the oracle (C restatement) and of the compiled reference driver.

Test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from x3dcore2_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "libe8oracle.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libe8ref.so")
REF_TIMING_LIB = os.path.join(ORACLE_DIR, "_ref", "libe8ref_timing.so")
SCENEGEN_LIB = os.path.join(ORACLE_DIR, "libe8scenegen.so")
# The reference checkout: E8G_REFERENCE_ROOT, by default /root/reference. Where there is none, the
# unmodified copy of its corelib sources that `make -C oracle ship` puts in the git-ignored
# reference install folder (baseline/_ref) stands in for it.
REFERENCE_ROOT = os.environ.get("E8G_REFERENCE_ROOT", "/root/reference")
SHIPPED_ROOT = os.path.join(ROOT, "baseline", "_ref")


def reference_root():
    """The reference checkout, else the shipped copy, else None."""
    for r in (REFERENCE_ROOT, SHIPPED_ROOT):
        if os.path.isfile(os.path.join(r, "corelib", "src", "renderer.cpp")):
            return r
    return None


def reference_src():
    r = reference_root()
    return os.path.join(r, "corelib", "src") if r else None


def reference_testdata(name):
    """A folder of the reference's testdata/ (checkout or shipped copy), or None."""
    for r in (REFERENCE_ROOT, SHIPPED_ROOT):
        d = os.path.join(r, "testdata", name)
        if os.path.isdir(d):
            return d
    return None


def build_reference():
    subprocess.run(["make", "-s", "-j2", "-C", ORACLE_DIR, "ref"], check=True)


class OHit(C.Structure):
    _fields_ = [("t", C.c_float), ("mesh", C.c_int32), ("tri", C.c_int32), ("b1", C.c_float),
                ("b2", C.c_float), ("vertex", C.c_float * 3), ("normal", C.c_float * 3)]


class OPolicy(C.Structure):
    _fields_ = [("max_depth", C.c_uint32), ("rr_start", C.c_uint32), ("rr_prob", C.c_float),
                ("bdpt_max_len", C.c_uint32)]


REF_POLICY = OPolicy(0, 2, 0.5, 8)
LT2_POLICY = OPolicy(0, 1, 0.5, 8)  # bidirect_lt2: Russian roulette from depth 1 (pathtracer.cpp:705)


def ref_policy(mode):
    """The reference's own policy for a tracer mode (what e8g_default_params sets)."""
    return LT2_POLICY if mode == abi.MODE_REF_LT2 else REF_POLICY

_P = C.c_void_p
_U = C.c_uint32


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "all"], check=True)


_oracle = None


def oracle():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_LIB):
            build_oracle()
        lib = C.CDLL(ORACLE_LIB)
        sig = {
            "o_scene_create": (_P, [C.POINTER(abi.SceneDesc)]),
            "o_scene_free": (None, [_P]),
            "o_bvh_stats": (None, [_P, _P, _P, _P]),
            "o_trace_closest": (None, [_P, _P, _U, C.c_int, _P]),
            "o_trace_any": (None, [_P, _P, _P, _P, _U, C.c_int, _P]),
            "o_trace_closest_counts": (None, [_P, _P, _U, _P, _P]),
            "o_camera_rays": (None, [_P, _U, _U, _P]),
            "o_render_paths": (None, [_P, _U, _U, C.c_uint64, C.POINTER(OPolicy), _U, _U, _P, _P,
                                      _U, _P, C.c_int]),
            "o_render": (None, [_P, _U, _U, C.c_uint64, C.POINTER(OPolicy), _U, _U, _U, _U, _U,
                                _U, _U, _U, _P, C.c_int]),
            "o_path_seed": (_U, [C.c_uint64, _U, _U]),
            "o_firefly_add": (None, [_P, _U, _U, _P]),
            "o_composite": (None, [_P, _U, _U, _U, C.c_int, C.c_float, _P]),
            "o_transform_mesh": (C.c_int, [_P, _P, _P, _U, _P, _P]),
            "o_render_task": (None, [_P, _U, C.POINTER(OPolicy), _U, _U, _U, C.c_int, _U, _P]),
            "o_minstd_draws": (None, [_U, _U, _P]),
            "o_philox_draws": (None, [C.c_uint64, _U, _U, _U, _P]),
            "o_bsdf_eval": (None, [_P, C.c_int32, _P, _P, _P, _P]),
            "o_bsdf_sample": (None, [_P, C.c_int32, _U, _P, _P, _U, _P, _P]),
            "o_path_gradient_f64": (None, [_P, C.c_uint64, C.POINTER(OPolicy), _U, _U, _U, _U, _P,
                                           _P, _P, _P]),
            "o_image_gradient_f64": (None, [_P, C.c_uint64, C.POINTER(OPolicy), _U, _U, _U, _P, _P, _P,
                                            C.c_int]),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _oracle = lib
    return _oracle


_scenegen = None


def scenegen():
    """The seeded scene generators built on their own (oracle/libe8scenegen.so, from the same
    source as the GPU library's), for processes that time the reference on the host cores and
    must not map the GPU library. Pass it as `lib=` to x3dcore2_gb300.scene's generators."""
    global _scenegen
    if _scenegen is None:
        if not os.path.exists(SCENEGEN_LIB):
            subprocess.run(["make", "-s", "-C", ORACLE_DIR, "gen"], check=True)
        _scenegen = abi.load(SCENEGEN_LIB)
    return _scenegen


_refs = {}


def reference_available():
    return os.path.exists(REF_LIB)


def reference(timing=False):
    path = REF_TIMING_LIB if timing else REF_LIB
    if path not in _refs:
        lib = C.CDLL(path)
        sig = {
            "r_scene_create": (_P, [C.POINTER(abi.SceneDesc)]),
            "r_scene_free": (None, [_P]),
            "r_trace_closest": (None, [_P, _P, _U, C.c_int, _P, _P, _P, _P, _P]),
            "r_trace_any": (None, [_P, _P, _P, _P, _U, C.c_int, _P]),
            "r_camera_rays": (None, [_P, _U, _U, _P]),
            "r_render_paths": (None, [_P, _U, _U, _U, _P, _P, _U, _P]),
            "r_render": (C.c_double, [_P, _U, _U, _U, _U, _U, _P, _P, C.c_int]),
            "r_composite": (None, [_P, _U, _U, _U, C.c_int, C.c_float, _P]),
            "r_transform_mesh": (C.c_int, [_P, _P, _P, _U, _P, _P]),
            "r_obj_load": (C.c_int, [C.c_char_p, _P, _P, _P, _P, _P, _P, C.c_char_p, _U]),
            "r_bsdf_eval": (None, [_P, C.c_int32, _P, _P, _P, _P]),
            "r_bsdf_sample": (None, [_P, C.c_int32, _U, _P, _P, _U, _P, _P]),
            "r_minstd_draws": (None, [_U, _U, _P]),
            "r_bvh_num_nodes": (_U, [_P]),
            "r_bvh_max_depth": (_U, [_P]),
            "r_uv_sphere": (_U, [C.c_float, _U, C.c_int, _P, _P, _P]),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _refs[path] = lib
    return _refs[path]


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def rays_array(o, d):
    """(n, 6) float32 array laid out like e8g_ray."""
    a = np.empty((len(o), 6), dtype=np.float32)
    a[:, :3] = o
    a[:, 3:] = d
    return a


class OracleScene:
    def __init__(self, scene):
        self.scene = scene
        self.lib = oracle()
        self.h = self.lib.o_scene_create(C.byref(scene.desc))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.o_scene_free(self.h)
            self.h = None

    def camera_rays(self, w, h):
        out = np.empty((w * h, 6), dtype=np.float32)
        self.lib.o_camera_rays(self.h, w, h, ptr(out))
        return out

    def trace_closest(self, rays, use_bvh=True):
        n = len(rays)
        hits = (OHit * max(1, n))()
        self.lib.o_trace_closest(self.h, ptr(rays), n, int(use_bvh), hits)
        t = np.array([hits[i].t for i in range(n)], dtype=np.float32)
        mesh = np.array([hits[i].mesh for i in range(n)], dtype=np.int32)
        tri = np.array([hits[i].tri for i in range(n)], dtype=np.int32)
        b = np.array([(hits[i].b1, hits[i].b2) for i in range(n)], dtype=np.float32).reshape(n, 2)
        vtx = np.array([list(hits[i].vertex) for i in range(n)], dtype=np.float32).reshape(n, 3)
        nrm = np.array([list(hits[i].normal) for i in range(n)], dtype=np.float32).reshape(n, 3)
        return dict(t=t, mesh=mesh, tri=tri, b=b, vertex=vtx, normal=nrm)

    def trace_any(self, rays, tmin, tmax, use_bvh=True):
        n = len(rays)
        out = np.zeros(n, dtype=np.uint8)
        self.lib.o_trace_any(self.h, ptr(rays), ptr(np.ascontiguousarray(tmin, np.float32)),
                             ptr(np.ascontiguousarray(tmax, np.float32)), n, int(use_bvh), ptr(out))
        return out

    def counts(self, rays):
        nodes, tris = C.c_uint64(), C.c_uint64()
        self.lib.o_trace_closest_counts(self.h, ptr(rays), len(rays), C.byref(nodes), C.byref(tris))
        return nodes.value, tris.value

    def render_paths(self, mode, w, h, pixels, seeds, policy=None, rng=abi.RNG_MINSTD,
                     seed=0, threads=8):
        policy = ref_policy(mode) if policy is None else policy
        pixels = np.ascontiguousarray(pixels, np.uint32)
        seeds = np.ascontiguousarray(seeds, np.uint32)
        out = np.zeros((len(pixels), 3), dtype=np.float32)
        self.lib.o_render_paths(self.h, mode, rng, seed, C.byref(policy), w, h, ptr(pixels),
                                ptr(seeds), len(pixels), ptr(out), threads)
        return out

    def render(self, mode, w, h, spp, seed=1, policy=None, rng=abi.RNG_MINSTD, offset=0,
               crop=None, threads=8):
        policy = ref_policy(mode) if policy is None else policy
        x0, y0, x1, y1 = crop if crop else (0, 0, w, h)
        out = np.zeros(((y1 - y0) * (x1 - x0), 4), dtype=np.float32)
        self.lib.o_render(self.h, mode, rng, seed, C.byref(policy), w, h, spp, offset, x0, y0, x1,
                          y1, ptr(out), threads)
        return out.reshape(y1 - y0, x1 - x0, 4)

    def image_gradient(self, seed, policy, w, h, spp, dl, threads=8):
        """FP64 path-replay gradient of the MIS image (Philox streams) under the upstream image
        gradient dl (h, w, 3): (d_albedo (materials, 3), d_roughness (materials,))."""
        nm = self.scene.desc.num_materials
        da = np.zeros(nm * 3, np.float64)
        dr = np.zeros(nm, np.float64)
        dl = np.ascontiguousarray(dl, np.float32).reshape(-1)
        self.lib.o_image_gradient_f64(self.h, seed, C.byref(policy), w, h, spp, ptr(dl), ptr(da), ptr(dr), threads)
        return da.reshape(nm, 3), dr

    def render_task(self, mode, w, h, spp, firefly=False, task_seed=33, policy=None):
        """pt_image_renderer::render with one task: the reference's own sequential stream."""
        policy = ref_policy(mode) if policy is None else policy
        out = np.zeros((w * h, 4), dtype=np.float32)
        self.lib.o_render_task(self.h, mode, C.byref(policy), w, h, spp, int(firefly), task_seed, ptr(out))
        return out.reshape(h, w, 4)

    def bsdf_eval(self, m, n, o, i):
        f = np.zeros(3, np.float32)
        self.lib.o_bsdf_eval(self.h, m, ptr(np.asarray(n, np.float32)), ptr(np.asarray(o, np.float32)),
                             ptr(np.asarray(i, np.float32)), ptr(f))
        return f

    def bsdf_sample(self, m, seed, n, o, count):
        d = np.zeros((count, 3), np.float32)
        p = np.zeros(count, np.float32)
        self.lib.o_bsdf_sample(self.h, m, seed, ptr(np.asarray(n, np.float32)),
                               ptr(np.asarray(o, np.float32)), count, ptr(d), ptr(p))
        return d, p

    def bvh_stats(self):
        a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self.lib.o_bvh_stats(self.h, C.byref(a), C.byref(b), C.byref(c))
        return dict(nodes=a.value, max_depth=b.value, leaves=c.value)


def firefly_add(est, acc):
    """The reference's firefly clamp on one sample image est (h, w, 3), added to acc in place."""
    est = np.ascontiguousarray(est, np.float32)
    assert acc.dtype == np.float32 and acc.flags.c_contiguous and acc.shape == est.shape
    oracle().o_firefly_add(ptr(est), est.shape[1], est.shape[0], ptr(acc))


def composite(rgba, tonemap, auto_exposure=True, exposure=1.0, lib=None):
    """The compositors on a float (h, w, 4) image: the oracle's restatement, or the compiled
    reference when lib is the reference library."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    h, w = rgba.shape[:2]
    out = np.zeros((h, w, 4), np.uint8)
    fn = (lib or oracle())
    f = fn.r_composite if lib is not None else fn.o_composite
    f(ptr(rgba), w, h, tonemap, int(auto_exposure), exposure, ptr(out))
    return out


def transform_mesh(m, pos, nrm, lib=None):
    """trimesh::transform of (n, 3) vertex and normal arrays by the row-major 4x4 matrix m: the
    oracle's restatement, or the compiled reference when lib is the reference library. Returns
    (positions, normals), or None where the reference throws (singular matrix)."""
    m = np.ascontiguousarray(m, np.float32).reshape(16)
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    po = np.zeros_like(pos)
    no = np.zeros_like(nrm)
    f = lib.r_transform_mesh if lib is not None else oracle().o_transform_mesh
    if not f(ptr(m), ptr(pos), ptr(nrm), len(pos), ptr(po), ptr(no)):
        return None
    return po, no


def ref_obj_load(path, lib):
    """wavefront_obj::load_geometry of the compiled reference: dict(pos, nrm, uv, tris), or the
    message of the exception it throws (a str)."""
    nv, nt = C.c_uint32(0), C.c_uint32(0)
    err = C.create_string_buffer(512)
    p = str(path).encode()
    if not lib.r_obj_load(p, C.byref(nv), C.byref(nt), None, None, None, None, err, len(err)):
        return err.value.decode(errors="replace")
    pos = np.zeros((nv.value, 3), np.float32)
    nrm = np.zeros((nv.value, 3), np.float32)
    uv = np.zeros((nv.value, 2), np.float32)
    tris = np.zeros((nt.value, 3), np.uint32)
    ok = lib.r_obj_load(p, C.byref(nv), C.byref(nt), ptr(pos), ptr(nrm), ptr(uv), ptr(tris), err, len(err))
    assert ok
    return dict(pos=pos, nrm=nrm, uv=uv, tris=tris)


class RefScene:
    """The compiled, unmodified reference, driven through its own C++ API."""

    def __init__(self, scene, timing=False):
        self.scene = scene
        self.lib = reference(timing)
        self.h = self.lib.r_scene_create(C.byref(scene.desc))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.r_scene_free(self.h)
            self.h = None

    def camera_rays(self, w, h):
        out = np.empty((w * h, 6), dtype=np.float32)
        self.lib.r_camera_rays(self.h, w, h, ptr(out))
        return out

    def trace_closest(self, rays, use_bvh=True):
        n = len(rays)
        t = np.zeros(n, np.float32)
        mesh = np.zeros(n, np.int32)
        tri = np.zeros(n, np.int32)
        vtx = np.zeros((n, 3), np.float32)
        nrm = np.zeros((n, 3), np.float32)
        self.lib.r_trace_closest(self.h, ptr(rays), n, int(use_bvh), ptr(t), ptr(mesh), ptr(tri),
                                 ptr(vtx), ptr(nrm))
        return dict(t=t, mesh=mesh, tri=tri, vertex=vtx, normal=nrm)

    def trace_any(self, rays, tmin, tmax, use_bvh=True):
        n = len(rays)
        out = np.zeros(n, dtype=np.uint8)
        self.lib.r_trace_any(self.h, ptr(rays), ptr(np.ascontiguousarray(tmin, np.float32)),
                             ptr(np.ascontiguousarray(tmax, np.float32)), n, int(use_bvh), ptr(out))
        return out

    def render_paths(self, mode, w, h, pixels, seeds):
        pixels = np.ascontiguousarray(pixels, np.uint32)
        seeds = np.ascontiguousarray(seeds, np.uint32)
        out = np.zeros((len(pixels), 3), dtype=np.float32)
        self.lib.r_render_paths(self.h, mode, w, h, ptr(pixels), ptr(seeds), len(pixels), ptr(out))
        return out

    def render(self, mode, w, h, spp, threads, firefly=False):
        out = np.zeros((w * h, 4), dtype=np.float32)
        taken = C.c_uint32()
        secs = self.lib.r_render(self.h, mode, w, h, spp, threads, ptr(out), C.byref(taken), int(firefly))
        return out.reshape(h, w, 4), secs, taken.value

    def bsdf_eval(self, m, n, o, i):
        f = np.zeros(3, np.float32)
        self.lib.r_bsdf_eval(self.h, m, ptr(np.asarray(n, np.float32)), ptr(np.asarray(o, np.float32)),
                             ptr(np.asarray(i, np.float32)), ptr(f))
        return f

    def bsdf_sample(self, m, seed, n, o, count):
        d = np.zeros((count, 3), np.float32)
        p = np.zeros(count, np.float32)
        self.lib.r_bsdf_sample(self.h, m, seed, ptr(np.asarray(n, np.float32)),
                               ptr(np.asarray(o, np.float32)), count, ptr(d), ptr(p))
        return d, p
