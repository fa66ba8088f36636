"""Scene descriptions on the host: generated scenes and scenes built from numpy arrays.

A scene mirrors what the reference loads into its containers: a list of world-space triangle
meshes (corelib trimesh, ascending object id), their material ids, the material table, the area
lights (ascending object id) and the pinhole camera.
"""
import ctypes as C

import numpy as np

from . import abi


class Scene:
    """Owns numpy arrays and the SceneDesc that points into them."""

    def __init__(self, voff, toff, mesh_mat, pos, nrm, tris, materials, lights, camera):
        self.voff = np.ascontiguousarray(voff, dtype=np.uint32)
        self.toff = np.ascontiguousarray(toff, dtype=np.uint32)
        self.mesh_mat = np.ascontiguousarray(mesh_mat, dtype=np.int32)
        self.pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        self.nrm = np.ascontiguousarray(nrm, dtype=np.float32).reshape(-1, 3)
        self.tris = np.ascontiguousarray(tris, dtype=np.uint32).reshape(-1, 3)
        self.materials = (abi.Material * max(1, len(materials)))(*materials)
        self.num_materials = len(materials)
        self.lights = (abi.Light * max(1, len(lights)))(*lights)
        self.num_lights = len(lights)
        self.camera = camera
        self.desc = abi.SceneDesc()
        d = self.desc
        d.num_meshes = len(self.mesh_mat)
        d.mesh_vert_offset = self.voff.ctypes.data_as(C.POINTER(C.c_uint32))
        d.mesh_tri_offset = self.toff.ctypes.data_as(C.POINTER(C.c_uint32))
        d.mesh_material = self.mesh_mat.ctypes.data_as(C.POINTER(C.c_int32))
        d.positions = self.pos.ctypes.data_as(C.POINTER(C.c_float))
        d.normals = self.nrm.ctypes.data_as(C.POINTER(C.c_float))
        d.triangles = self.tris.ctypes.data_as(C.POINTER(C.c_uint32))
        d.num_materials = self.num_materials
        d.materials = C.cast(self.materials, C.POINTER(abi.Material))
        d.num_lights = self.num_lights
        d.lights = C.cast(self.lights, C.POINTER(abi.Light))
        d.camera = camera

    @property
    def num_tris(self):
        return int(self.toff[-1])

    def tri_mesh(self):
        """Mesh index of every global triangle."""
        return np.repeat(np.arange(len(self.mesh_mat), dtype=np.int32), np.diff(self.toff))

    def world_triangles(self):
        """(T, 3, 3) float32 vertex positions of every triangle."""
        base = np.repeat(self.voff[:-1], np.diff(self.toff)).astype(np.int64)
        idx = self.tris.astype(np.int64) + base[:, None]
        return self.pos[idx]

    def with_materials(self, materials):
        return Scene(self.voff, self.toff, self.mesh_mat, self.pos, self.nrm, self.tris,
                     list(materials), list(self.lights[:self.num_lights]), self.camera)

    def material_list(self):
        return [self.materials[i] for i in range(self.num_materials)]


def from_desc(desc):
    """Copy a SceneDesc (e.g. one a generator filled) into an owning Scene."""
    nm = desc.num_meshes
    voff = np.ctypeslib.as_array(desc.mesh_vert_offset, shape=(nm + 1,)).copy()
    toff = np.ctypeslib.as_array(desc.mesh_tri_offset, shape=(nm + 1,)).copy()
    nv, nt = int(voff[-1]), int(toff[-1])
    mesh_mat = np.ctypeslib.as_array(desc.mesh_material, shape=(nm,)).copy()
    pos = np.ctypeslib.as_array(desc.positions, shape=(nv * 3,)).copy()
    nrm = np.ctypeslib.as_array(desc.normals, shape=(nv * 3,)).copy()
    tris = np.ctypeslib.as_array(desc.triangles, shape=(nt * 3,)).copy()
    mats = [abi.Material.from_buffer_copy(desc.materials[i]) for i in range(desc.num_materials)]
    lights = [abi.Light.from_buffer_copy(desc.lights[i]) for i in range(desc.num_lights)]
    cam = abi.Camera.from_buffer_copy(desc.camera)
    return Scene(voff, toff, mesh_mat, pos, nrm, tris, mats, lights, cam)


class Mesh:
    """One triangle mesh on the host: positions and normals (n, 3), texcoords (n, 2), triangles (m, 3)."""

    def __init__(self, pos, nrm, tris, uv=None):
        self.pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        self.nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
        self.tris = np.ascontiguousarray(tris, np.uint32).reshape(-1, 3)
        self.uv = np.zeros((len(self.pos), 2), np.float32) if uv is None else np.asarray(uv, np.float32)


def _take_mesh(lib, h):
    try:
        d = abi.MeshData()
        abi.check(lib.e8g_host_mesh_data(h, C.byref(d)), what="e8g_host_mesh_data")
        nv, nt = d.num_vertices, d.num_triangles
        arr = np.ctypeslib.as_array
        return Mesh(arr(d.positions, (nv * 3,)).copy() if nv else np.zeros(0, np.float32),
                    arr(d.normals, (nv * 3,)).copy() if nv else np.zeros(0, np.float32),
                    arr(d.triangles, (nt * 3,)).copy() if nt else np.zeros(0, np.uint32),
                    arr(d.texcoords, (nv * 2,)).reshape(-1, 2).copy() if nv else None)
    finally:
        lib.e8g_host_mesh_free(h)


def load_obj(path=None, text=None, lib=None):
    """A Wavefront OBJ mesh read with the reference loader's rules (e8g_obj_load / e8g_obj_parse).
    Raises E8GError with the loader's message on a malformed file."""
    lib = lib or abi.load()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    if text is not None:
        raw = text.encode() if isinstance(text, str) else bytes(text)
        st = lib.e8g_obj_parse(raw, len(raw), C.byref(h), err, len(err))
    else:
        st = lib.e8g_obj_load(str(path).encode(), C.byref(h), err, len(err))
    if st != abi.E8G_OK:
        raise abi.E8GError(f"{abi.STATUS_NAMES.get(st, st)}: {err.value.decode(errors='replace')}")
    return _take_mesh(lib, h)


def from_meshes(meshes, mesh_material, materials, lights, camera):
    """A Scene of meshes in the given order (the reference path space's ascending object id)."""
    voff = np.concatenate([[0], np.cumsum([len(m.pos) for m in meshes])]).astype(np.uint32)
    toff = np.concatenate([[0], np.cumsum([len(m.tris) for m in meshes])]).astype(np.uint32)
    pos = np.concatenate([m.pos for m in meshes]) if meshes else np.zeros((0, 3), np.float32)
    nrm = np.concatenate([m.nrm for m in meshes]) if meshes else np.zeros((0, 3), np.float32)
    tris = np.concatenate([m.tris for m in meshes]) if meshes else np.zeros((0, 3), np.uint32)
    return Scene(voff, toff, mesh_material, pos, nrm, tris, list(materials), list(lights), camera)


def generate(kind, seed=1, level=0, num_tris=0, num_materials=0, amplitude=0.0,
             roughness_lo=0.0, roughness_hi=0.0, width=0, height=0, lib=None):
    """Run one of the native generators (host code; no GPU needed)."""
    lib = lib or abi.load()
    o = abi.GenOpts(kind=kind, seed=seed, level=level, num_tris=num_tris,
                    num_materials=num_materials, amplitude=amplitude, roughness_lo=roughness_lo,
                    roughness_hi=roughness_hi, width=width, height=height)
    h = C.c_void_p()
    abi.check(lib.e8g_gen_scene(C.byref(o), C.byref(h)), what="e8g_gen_scene")
    try:
        d = abi.SceneDesc()
        abi.check(lib.e8g_host_scene_desc(h, C.byref(d)), what="e8g_host_scene_desc")
        return from_desc(d)
    finally:
        lib.e8g_host_scene_free(h)


def cornell(width=256, height=256, **kw):
    """Cornell box: unit room, two rotated boxes, 0.25^2 light of radiance (17, 12, 4)."""
    return generate(abi.GEN_CORNELL, width=width, height=height, **kw)


def displaced_icosphere(level=8, seed=1, num_materials=512, width=1920, height=1080, **kw):
    """Displaced icosphere (20 * 4^level faces) on a ground plane with 4 quad lights."""
    return generate(abi.GEN_DISPLACED_ICO, seed=seed, level=level, num_materials=num_materials,
                    amplitude=kw.pop("amplitude", 0.05), width=width, height=height, **kw)


def soup(num_tris=1000, seed=1, width=256, height=256, **kw):
    """Random triangle soup inside an enclosing room with an area light."""
    return generate(abi.GEN_SOUP, seed=seed, num_tris=num_tris, width=width, height=height, **kw)


def furnace(res=30):
    """The reference's furnace sphere: inward uv_sphere r=10, Lambert 0.7, emission 1."""
    return generate(abi.GEN_FURNACE, level=res)


def material(kind, albedo=(0.8, 0.8, 0.8), roughness=0.0, ior=(1.5, 0.0), mix=(-1, -1),
             ratio=0.5):
    m = abi.Material()
    m.type = kind
    m.albedo[:] = list(albedo)
    m.roughness = roughness
    m.ior_re, m.ior_im = ior
    m.mix0, m.mix1 = mix
    m.ratio = ratio
    return m
